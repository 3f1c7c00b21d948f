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
/* evolution::Wedge: VecGeom/volumes/Wedge_Evolution.h                */
/* ================================================================== */

/* Wedge(angle, zeroangle) (source/Wedge_Evolution.cpp:17-99) */
static void wedge_init(or_wedge *w, double dphi, double sphi)
{
  w->a1x  = cos(sphi);
  w->a1y  = sin(sphi);
  w->a2x  = cos(sphi + dphi);
  w->a2y  = sin(sphi + dphi);
  w->n1x  = -sin(sphi);
  w->n1y  = cos(sphi);
  w->n2x  = sin(sphi + dphi);
  w->n2y  = -cos(sphi + dphi);
  w->dphi = dphi;
}

/* Wedge::IsOnSurfaceGeneric (Wedge_Evolution.h:341-354) */
static inline int wedge_on_surface(double ax, double ay, double nx, double ny, v3 p)
{
  if (!(ax * p.x + ay * p.y >= 0.)) return 0;
  return fabs(nx * p.x + ny * p.y) < kTolerance;
}

/* Wedge::GenericKernelForContainsAndInside (Wedge_Evolution.h:306-339) */
static void wedge_ci(const or_wedge *w, v3 p, int forInside, int *cin, int *cout)
{
  double startCheck = (-p.x * w->a1y + p.y * w->a1x);
  double endCheck   = (-w->a2x * p.y + w->a2y * p.x);
  *cout             = startCheck < 0.;
  if (w->dphi < kPi)
    *cout = *cout || endCheck < 0.;
  else
    *cout = *cout && endCheck < 0.;
  if (forInside) {
    int onSurface = wedge_on_surface(w->a1x, w->a1y, w->n1x, w->n1y, p) ||
                    wedge_on_surface(w->a2x, w->a2y, w->n2x, w->n2y, p);
    *cout = *cout && !onSurface;
    *cin  = !onSurface && !*cout;
  }
}

/* Wedge::Contains (Wedge_Evolution.h:296-303) */
static inline int wedge_contains(const or_wedge *w, v3 p)
{
  int cin = 0, cout = 0;
  wedge_ci(w, p, 0, &cin, &cout);
  return !cout;
}

/* Wedge::SafetyToIn (Wedge_Evolution.h:374-391) */
static double wedge_safe_in(const or_wedge *w, v3 p)
{
  double dist1 = p.x * w->n1x + p.y * w->n1y;
  double dist2 = p.x * w->n2x + p.y * w->n2y;
  if (w->dphi < kPi) return or_max(-1 * dist1, -1 * dist2);
  return or_min(-1 * dist1, -1 * dist2);
}

/* Wedge::SafetyToOut (Wedge_Evolution.h:356-372) */
static double wedge_safe_out(const or_wedge *w, v3 p)
{
  double dist1 = p.x * w->n1x + p.y * w->n1y;
  double dist2 = p.x * w->n2x + p.y * w->n2y;
  if (w->dphi < kPi) return or_min(dist1, dist2);
  return or_max(dist1, dist2);
}

/* ================================================================== */
/* Tube (UniversalTube): kernel/TubeImplementation.h                  */
/* ================================================================== */

/* TubeStruct constructor + CalculateCached (TubeStruct.h:43-72, 153-175): the raw
 * (sphi, dphi) are kept (the constructor does not call SetAndCheck*PhiAngle); the phi
 * treatment is on when dphi < 2 pi (TubeTypes.h:91-98, UniversalTube) */
static int tube_init(or_tube *t, const double *a, char *err, int errlen)
{
  t->rmin = a[0] < 0.0 ? 0.0 : a[0];
  t->rmax = a[1];
  t->z    = a[2];
  t->sphi = a[3];
  t->dphi = a[4];
  if (!(t->rmax > t->rmin && t->z > 0 && t->dphi > 0)) {
    set_err(err, errlen, "tube: needs rmax > rmin, dz > 0 and dphi > 0");
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
  wedge_init(&t->w, t->dphi, t->sphi);
  return 0;
}

static inline int tube_has_phi(const or_tube *t) { return t->dphi < kTwoPi; } /* checkPhiTreatment */

/* TubeUtilities::PointInCyclicalSector<..., onSurfaceT = false> (TubeImplementation.h:58-101);
 * UniversalTube decides "smaller than pi" at run time (dphi <= M_PI) */
static int tube_in_sector(const or_tube *t, double x, double y, int includeSurface)
{
  double startCheck = (-x * t->alongphi1y + y * t->alongphi1x);
  double endCheck   = (-t->alongphi2x * y + t->alongphi2y * x);
  double tol        = includeSurface ? -kHalfTolerance : kHalfTolerance;
  if (t->dphi <= kPi) return (startCheck >= tol) && (endCheck >= tol);
  return (startCheck >= tol) || (endCheck >= tol);
}

/* TubeUtilities::CircleTrajectoryIntersection (TubeImplementation.h:103-160) */
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
    if (!*ok) return;
    if (tube_has_phi(t)) {
      double hitx = pos.x + *dist * dir.x;
      double hity = pos.y + *dist * dir.y;
      *ok &= tube_in_sector(t, hitx, hity, 1);
    }
  }
}

/* TubeUtilities::PhiPlaneTrajectoryIntersection (TubeImplementation.h:249-301) */
static void tube_phi_plane(const or_tube *t, double alongX, double alongY, double normalX, double normalY, v3 pos,
                           v3 dir, int posdir, int insector, double *dist, int *ok)
{
  double dirDotNorm = dir.x * normalX + dir.y * normalY;
  double dirDotXY;
  *ok      = insector ? (dirDotNorm > 0.) : (dirDotNorm < 0.);
  dirDotXY = (dir.y * alongX - dir.x * alongY);
  *dist    = (alongY * pos.x - alongX * pos.y) / NonZero(dirDotXY);
  *ok &= (*dist * fabs(dirDotNorm)) > -kHalfTolerance;
  if (insector) {
    double hitx = pos.x + *dist * dir.x;
    double hity = pos.y + *dist * dir.y;
    double hitz = pos.z + *dist * dir.z;
    double r2   = hitx * hitx + hity * hity;
    *ok &= fabs(hitz) <= t->tolOz && (r2 >= t->tolOrmin2) && (r2 <= t->tolOrmax2);
    if (posdir) *ok = *ok && (hitx * alongX + hity * alongY) > 0.;
  } else if (posdir) {
    double hitx = pos.x + *dist * dir.x;
    double hity = pos.y + *dist * dir.y;
    *ok         = *ok && (hitx * alongX + hity * alongY) >= 0.;
  }
}

/* TubeUtilities::PhiPlaneSafety<inside = false> (TubeImplementation.h:210-247), UniversalTube */
static double tube_phi_safety(const or_tube *t, v3 pos)
{
  double safety = t->dphi > kPi ? sqrt(pos.x * pos.x + pos.y * pos.y) : kInfLength;
  double phi1   = pos.x * t->alongphi1y - pos.y * t->alongphi1x; /* PerpDist2D */
  double phi2;
  if (phi1 > -kHalfTolerance && phi1 < safety) safety = phi1;
  phi2 = pos.x * t->alongphi2y - pos.y * t->alongphi2x;
  phi2 *= -1;
  if (phi2 > -kHalfTolerance && phi2 < safety) safety = phi2;
  return safety;
}

/* DistanceToInKernel (TubeImplementation.h:504-681), rmin and phi treatment at run time */
static double tube_dist_in_kernel(const or_tube *t, v3 p, v3 d)
{
  int done = 0, inside, okz, onsurf, ok_rmax, ok_rmin, ok_phi;
  double distance = kInfLength, distz, rsq, rdotn, hitx, hity, r2, invnsq, b, crmax, dist_rmax, dist_rmin, dist_phi;
  const int hasrmin = t->rmin > 0;
  const int hasphi  = tube_has_phi(t);

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
  if (hasphi && inside) inside &= tube_in_sector(t, p.x, p.y, 0);
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
  if (hasphi && okz) okz &= tube_in_sector(t, hitx, hity, 1);
  if (!done && okz) distance = distz;
  done |= okz;

  {
    /* IsMovingInsideTubeSurface (TubeImplementation.h:317-343) */
    const double rho = p.x * p.x + p.y * p.y;
    onsurf = (rho >= t->tolIrmax2) && (rho <= t->tolOrmax2) && (fabs(p.z) < (t->z + kTolerance)) &&
             (d.x * p.x + d.y * p.y + d.z * 0. <= 0.);
    if (hasrmin)
      onsurf |= (rho >= t->tolOrmin2) && (rho <= t->tolIrmin2) && (fabs(p.z) < (t->z + kTolerance)) &&
                (d.x * -p.x + d.y * -p.y + d.z * 0. <= 0.);
  }
  if (hasphi) onsurf = onsurf && tube_in_sector(t, p.x, p.y, 1);
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

  if (hasphi) { /* SectorType of UniversalTube is unknown: both planes, positive-direction check */
    tube_phi_plane(t, t->alongphi1x, t->alongphi1y, t->w.n1x, t->w.n1y, p, d, 1, 1, &dist_phi, &ok_phi);
    ok_phi &= dist_phi < distance;
    if (!done && ok_phi) distance = dist_phi;
    done |= ok_phi;
    tube_phi_plane(t, t->alongphi2x, t->alongphi2y, t->w.n2x, t->w.n2y, p, d, 1, 1, &dist_phi, &ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
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
  int done = 0, ok_rmin, ok_rmax, ok_phi;
  double distance = -1., distz, rsq, rdotn, crmax, crmin, invdirz, invnsq, b, dist_rmin, dist_rmax, dist_phi;
  const int hasrmin = t->rmin > 0;
  const int hasphi  = tube_has_phi(t);

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
  if (hasphi) {
    int cin = 0, cout = 0;
    wedge_ci(&t->w, p, 1, &cin, &cout);
    done |= cout;
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

  if (hasphi) { /* angle bigger than pi or unknown: positive-direction check on both planes */
    tube_phi_plane(t, t->alongphi1x, t->alongphi1y, t->w.n1x, t->w.n1y, p, d, 1, 0, &dist_phi, &ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
    tube_phi_plane(t, t->alongphi2x, t->alongphi2y, t->w.n2x, t->w.n2y, p, d, 1, 0, &dist_phi, &ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  return distance;
}

/* SafetyToInOld (TubeImplementation.h:912-938; TUBE_SAFETY_OLD is defined at line 14) */
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
  if (tube_has_phi(t)) {
    int insector = tube_in_sector(t, p.x, p.y, 0);
    double safephi;
    if (insector) return safety;
    safephi = tube_phi_safety(t, p);
    if (!insector && safephi < kInfLength && safephi > safety) safety = safephi;
  }
  return safety;
}

/* SafetyToOutOld (TubeImplementation.h:940-966) */
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
  if (tube_has_phi(t)) {
    double safephi = wedge_safe_out(&t->w, p);
    if (safephi < safety) safety = safephi;
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
    if (*cout) return;
  }
  if (tube_has_phi(t)) {
    int cinphi = 0, coutphi = 0;
    wedge_ci(&t->w, p, forinside, &cinphi, &coutphi);
    *cout |= coutphi;
    if (forinside) *cin &= cinphi;
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

/* UnplacedTube::Extent (source/UnplacedTube.cpp:214-266) */
static void tube_extent(const or_tube *t, v3 *mn, v3 *mx)
{
  double Rin, Cx, Dx, Cy, Dy, Ax, Bx, Ay, By, temp;
  int phi0out, phi90out, phi180out, phi270out;
  *mn = v3_make(-t->rmax, -t->rmax, -t->z);
  *mx = v3_make(t->rmax, t->rmax, t->z);
  if (t->dphi == kTwoPi) return;
  Rin       = 0.5 * (t->rmax + t->rmin);
  phi0out   = !wedge_contains(&t->w, v3_make(Rin, 0, 0));
  phi90out  = !wedge_contains(&t->w, v3_make(0, Rin, 0));
  phi180out = !wedge_contains(&t->w, v3_make(-Rin, 0, 0));
  phi270out = !wedge_contains(&t->w, v3_make(0, -Rin, 0));
  if (!(phi0out || phi90out || phi180out || phi270out)) return;
  Cx = t->rmax * cos(t->sphi);
  Dx = t->rmax * cos(t->sphi + t->dphi);
  Cy = t->rmax * sin(t->sphi);
  Dy = t->rmax * sin(t->sphi + t->dphi);
  if (phi0out) mx->x = or_max(Cx, Dx);
  if (phi90out) mx->y = or_max(Cy, Dy);
  if (phi180out) mn->x = or_min(Cx, Dx);
  if (phi270out) mn->y = or_min(Cy, Dy);
  if (t->dphi >= kPi) return;
  Ax = t->rmin * cos(t->sphi);
  Bx = t->rmin * cos(t->sphi + t->dphi);
  Ay = t->rmin * sin(t->sphi);
  By = t->rmin * sin(t->sphi + t->dphi);
  temp  = or_max(Ax, Bx);
  mx->x = temp > mx->x ? temp : mx->x;
  temp  = or_max(Ay, By);
  mx->y = temp > mx->y ? temp : mx->y;
  temp  = or_min(Ax, Bx);
  mn->x = temp < mn->x ? temp : mn->x;
  temp  = or_min(Ay, By);
  mn->y = temp < mn->y ? temp : mn->y;
}

/* ================================================================== */
/* Cone (full phi): kernel/ConeImplementation.h, ConeUtilities.h      */
/* ================================================================== */

/* ConeStruct constructor + CalculateCached (ConeStruct.h:79-157, 414-426) */
static int cone_init(or_cone *c, const double *a, char *err, int errlen)
{
  double dphi = a[6], sphi = a[5];
  c->rmin1 = a[0] < 0.0 ? 0.0 : a[0];
  c->rmax1 = a[1];
  c->rmin2 = a[2] < 0.0 ? 0.0 : a[2];
  c->rmax2 = a[3];
  c->dz    = a[4];
  c->sphi  = a[5];
  c->o_rmin1 = a[0];
  c->o_rmax1 = a[1];
  c->o_rmin2 = a[2];
  c->o_rmax2 = a[3];
  if (!(dphi > 0)) {
    set_err(err, errlen, "cone: needs dphi > 0");
    return -1;
  }
  /* fPhiWedge(_dphi, _sphi), then SetAndCheckDPhiAngle(_dphi) and SetAndCheckSPhiAngle(_sphi)
   * (ConeStruct.h:321-360, 413-425): the wedge keeps the raw angles' vectors and takes the
   * checked delta; the along vectors use the checked angles */
  wedge_init(&c->w, dphi, sphi);
  c->dphi = dphi;
  if (dphi >= kTwoPi - 0.5 * kAngTolerance) {
    c->dphi = kTwoPi;
    c->sphi = 0;
  }
  c->w.dphi = c->dphi;
  if (sphi < 0)
    c->sphi = kTwoPi - fmod(fabs(sphi), kTwoPi);
  else
    c->sphi = fmod(sphi, kTwoPi);
  if (c->sphi + c->dphi > kTwoPi) c->sphi -= kTwoPi;
  c->alongphi1x = cos(c->sphi);
  c->alongphi1y = sin(c->sphi);
  c->alongphi2x = cos(c->sphi + c->dphi);
  c->alongphi2y = sin(c->sphi + c->dphi);
  c->originalRmax1 = c->rmax1;
  c->originalRmax2 = c->rmax2;
  if (c->rmin1 == c->rmax1) c->rmax1 += kConeTolerance;
  if (c->rmin2 == c->rmax2) c->rmax2 += kConeTolerance;
  c->sqRmin1    = c->rmin1 * c->rmin1;
  c->sqRmax1    = c->rmax1 * c->rmax1;
  c->sqRmin2    = c->rmin2 * c->rmin2;
  c->sqRmax2    = c->rmax2 * c->rmax2;
  c->tanRMin    = (c->rmin2 - c->rmin1) * 0.5 / c->dz;
  c->secRMin    = sqrt(1.0 + c->tanRMin * c->tanRMin);
  c->invSecRMin = 1. / NonZero(c->secRMin);
  c->tanRMax    = (c->rmax2 - c->rmax1) * 0.5 / c->dz;
  c->secRMax    = sqrt(1.0 + c->tanRMax * c->tanRMax);
  c->invSecRMax = 1. / NonZero(c->secRMax);
  c->innerSlope     = -(c->rmin1 - c->rmin2) / (2. * c->dz);
  c->outerSlope     = -(c->rmax1 - c->rmax2) / (2. * c->dz);
  c->innerOffset    = c->rmin2 - c->innerSlope * c->dz;
  c->outerOffset    = c->rmax2 - c->outerSlope * c->dz;
  c->innerTolerance = kConeTolerance * c->secRMin;
  c->outerTolerance = kConeTolerance * c->secRMax;
  if (c->rmin2 > c->rmin1) {
    c->innerConeApex     = 2 * c->dz * c->rmin1 / (c->rmin2 - c->rmin1);
    c->tanInnerApexAngle = c->rmin2 / (2 * c->dz + c->innerConeApex);
  } else {
    c->innerConeApex     = 2 * c->dz * c->rmin2 / NonZero(c->rmin1 - c->rmin2);
    c->tanInnerApexAngle = c->rmin1 / (2 * c->dz + c->innerConeApex);
  }
  if (c->rmin1 == 0. || c->rmin2 == 0.) c->innerConeApex = 0.;
  if (c->rmin1 == 0.) c->tanInnerApexAngle = c->rmin2 / (2 * c->dz);
  if (c->rmin2 == 0.) c->tanInnerApexAngle = c->rmin1 / (2 * c->dz);
  if (c->rmax2 > c->rmax1) {
    c->outerConeApex     = 2 * c->dz * c->rmax1 / (c->rmax2 - c->rmax1);
    c->tanOuterApexAngle = c->rmax2 / (2 * c->dz + c->outerConeApex);
  } else {
    c->outerConeApex     = 2 * c->dz * c->rmax2 / NonZero(c->rmax1 - c->rmax2);
    c->tanOuterApexAngle = c->rmax1 / (2 * c->dz + c->outerConeApex);
  }
  if (c->rmax1 == 0. || c->rmax2 == 0.) c->outerConeApex = 0.;
  if (c->rmax1 == 0.) c->tanOuterApexAngle = c->rmax2 / (2 * c->dz);
  if (c->rmax2 == 0.) c->tanOuterApexAngle = c->rmax1 / (2 * c->dz);
  c->zNormInner = c->tanRMin / NonZero(c->secRMin);
  c->zNormOuter = -c->tanRMax / NonZero(c->secRMax);
  c->tolIz      = c->dz - kHalfTolerance;
  c->tolOz      = c->dz + kHalfTolerance;
  return 0;
}

static inline int cone_has_rmin(const or_cone *c) { return c->rmin1 > 0 || c->rmin2 > 0; }

/* MakePlus/MinusTolerantSquare<true> (kernel/GenericKernels.h:65-82) */
static inline double plus_tol_sq(double x, double tol) { return x * (x + 2.0 * tol); }
static inline double minus_tol_sq(double x, double tol) { return fabs(x * (x - 2.0 * tol)); }

/* ConeUtilities::GetRadiusOfConeAtPoint (ConeUtilities.h:116-137) */
static inline double cone_radius(const or_cone *c, double z, int inner)
{
  if (inner) return c->rmin1 == c->rmin2 ? c->rmin1 : c->innerSlope * z + c->innerOffset;
  return c->originalRmax1 == c->originalRmax2 ? c->originalRmax1 : c->outerSlope * z + c->outerOffset;
}

static inline int cone_has_phi(const or_cone *c) { return c->dphi < kTwoPi; } /* ConeTypes.h:101-107 */

/* ConeUtilities::PointInCyclicalSector<..., onSurfaceT = false> (ConeUtilities.h:64-114),
 * UniversalCone: "smaller than pi" is dphi <= M_PI */
static int cone_in_sector(const or_cone *c, double x, double y, int includeSurface)
{
  double startCheck = (-x * c->alongphi1y) + (y * c->alongphi1x);
  double endCheck   = (-c->alongphi2x * y) + (c->alongphi2y * x);
  double tol        = includeSurface ? -kConeTolerance : kConeTolerance;
  if (c->dphi <= kPi) return (startCheck >= tol) && (endCheck >= tol);
  return (startCheck >= tol) || (endCheck >= tol);
}

/* ConeUtilities::PhiPlaneTrajectoryIntersection (ConeUtilities.h:155-204) */
static void cone_phi_plane(const or_cone *c, double alongX, double alongY, double normalX, double normalY, v3 pos,
                           v3 dir, int posdir, int insector, double *dist, int *ok)
{
  double dirDotXY;
  *dist = kInfLength;
  if (insector)
    *ok = ((dir.x * normalX) + (dir.y * normalY) > 0.);
  else
    *ok = ((dir.x * normalX) + (dir.y * normalY) < 0.);
  dirDotXY = (dir.y * alongX) - (dir.x * alongY);
  if (dirDotXY != 0) *dist = ((alongY * pos.x) - (alongX * pos.y)) / NonZero(dirDotXY);
  *ok &= *dist > -kConeTolerance;
  if (insector) {
    double hitx = pos.x + *dist * dir.x;
    double hity = pos.y + *dist * dir.y;
    double hitz = pos.z + *dist * dir.z;
    double r2   = (hitx * hitx) + (hity * hity);
    double innerRadIrTol = cone_radius(c, hitz, 1) + kTolerance;
    double outerRadIrTol = cone_radius(c, hitz, 0) - kTolerance;
    *ok &= fabs(hitz) <= c->tolIz && (r2 >= innerRadIrTol * innerRadIrTol) && (r2 <= outerRadIrTol * outerRadIrTol);
    if (posdir) *ok = *ok && ((hitx * alongX) + (hity * alongY)) > 0.;
  } else if (posdir) {
    double hitx = pos.x + *dist * dir.x;
    double hity = pos.y + *dist * dir.y;
    *ok         = *ok && ((hitx * alongX) + (hity * alongY)) >= 0.;
  }
}

/* ConeUtilities::GetNormal (ConeUtilities.h:206-238) */
static inline v3 cone_normal(const or_cone *c, v3 p, int inner)
{
  double rho = sqrt(v3_perp2(p));
  if (inner) {
    if ((c->rmin1 == c->rmin2) && (c->rmin1 != 0.)) return v3_make(-p.x, -p.y, 0.);
    return v3_make(-p.x, -p.y, c->zNormInner * (rho * c->secRMin));
  }
  if ((c->rmax1 == c->rmax2) && (c->rmax1 != 0.)) return v3_make(p.x, p.y, 0.);
  return v3_make(p.x, p.y, c->zNormOuter * (rho * c->secRMax));
}

/* ConeUtilities::IsOnConicalSurface (ConeUtilities.h:240-255) */
static inline int cone_on_surface(const or_cone *c, v3 p, int inner)
{
  const double rho      = v3_perp2(p);
  const double coneRad  = cone_radius(c, p.z, inner);
  const double coneRad2 = coneRad * coneRad;
  const double tol      = inner ? c->innerTolerance : c->outerTolerance;
  return (rho >= (coneRad2 - tol * coneRad)) && (rho <= (coneRad2 + tol * coneRad)) &&
         (fabs(p.z) < (c->dz + kConeTolerance));
}

/* ConeHelpers<double>::DetectIntersectionAndCalculateDistanceToConicalSurface (ConeUtilities.h:591-762) */
static int cone_conical(const or_cone *c, v3 p, v3 d, int fordistin, int inner, double *distance)
{
  int onsurf, ok = 0;
  v3 n;
  double pDotV2D, a, b, cc, b2, ac, d2, delta, newZ;
  *distance = kInfLength;
  onsurf    = cone_on_surface(c, p, inner);
  n         = cone_normal(c, p, inner);
  if (onsurf && fabs(v3_dot(d, n)) == 0.) return 0;
  if (onsurf) {
    int moving = fordistin ? (v3_dot(d, n) <= 0.) : (v3_dot(d, n) >= 0.);
    if (cone_has_phi(c)) moving = cone_in_sector(c, p.x, p.y, 1) && moving;
    if (moving) {
      *distance = 0.;
      return 1;
    }
  }
  pDotV2D = p.x * d.x + p.y * d.y;
  if (inner) {
    if (c->rmin1 == c->rmin2) {
      b  = pDotV2D;
      a  = v3_perp2(d);
      cc = v3_perp2(p) - c->rmin2 * c->rmin2;
    } else {
      double newPz, dirT;
      if (c->rmin2 > c->rmin1)
        newPz = (p.z + c->dz + c->innerConeApex) * c->tanInnerApexAngle;
      else
        newPz = (p.z - c->dz - c->innerConeApex) * c->tanInnerApexAngle;
      dirT = d.z * c->tanInnerApexAngle;
      a    = (d.x * d.x) + (d.y * d.y) - dirT * dirT;
      b    = pDotV2D - (newPz * dirT);
      cc   = v3_perp2(p) - (newPz * newPz);
    }
    b2 = b * b;
    ac = a * cc;
    if (b2 < ac) return 0;
    d2    = b2 - ac;
    delta = sqrt(d2);
    if (fordistin) {
      if (b >= 0.)
        *distance = (cc / NonZero(-b - delta));
      else
        *distance = (-b + delta) / NonZero(a);
    } else {
      if (b == 0. && delta == 0.) return 0;
      if (b >= 0.)
        *distance = (-b - delta) / NonZero(a);
      else
        *distance = (cc / NonZero(-b + delta));
    }
    if (*distance < 0.) return 0;
    newZ = p.z + (d.z * *distance);
    ok   = (fabs(newZ) < c->dz);
  } else {
    if (c->originalRmax1 == c->originalRmax2) {
      a  = v3_perp2(d);
      b  = pDotV2D;
      cc = (v3_perp2(p) - c->originalRmax2 * c->originalRmax2);
    } else {
      double newPz, dirT;
      if (c->originalRmax2 > c->originalRmax1)
        newPz = (p.z + c->dz + c->outerConeApex) * c->tanOuterApexAngle;
      else
        newPz = (p.z - c->dz - c->outerConeApex) * c->tanOuterApexAngle;
      dirT = d.z * c->tanOuterApexAngle;
      a    = d.x * d.x + d.y * d.y - dirT * dirT;
      b    = (pDotV2D - (newPz * dirT));
      cc   = (v3_perp2(p) - (newPz * newPz));
    }
    b2 = b * b;
    ac = a * cc;
    d2 = b2 - ac;
    if (d2 < 0) return 0;
    delta = sqrt(d2);
    if (fordistin) {
      if (b == 0. && delta == 0.) return 0;
      if (b > 0.)
        *distance = (-b - delta) / NonZero(a);
      else
        *distance = (cc / NonZero(-b + delta));
      newZ = p.z + (d.z * *distance);
      ok   = (fabs(newZ) < c->dz + kHalfTolerance);
    } else {
      if (b < 0.)
        *distance = (-b + delta) / NonZero(a);
      else
        *distance = (cc / NonZero(-b - delta));
      ok = *distance > 0.;
    }
    if (*distance < 0.) return 0;
  }
  if (cone_has_phi(c)) {
    double hitx = 0, hity = 0;
    if (*distance < kInfLength) {
      hitx = p.x + *distance * d.x;
      hity = p.y + *distance * d.y;
    }
    ok &= (cone_in_sector(c, hitx, hity, 1) && (*distance < kInfLength));
  }
  return ok;
}

/* DistanceToIn (ConeImplementation.h:117-255), full phi */
static double cone_dist_in(const or_cone *c, v3 p, v3 d)
{
  int done = 0, inside, okz, top, bot, ok;
  double distance = kInfLength, distz, outerRad, rsq, hitx, hity, r2, dr;
  const int hasrmin = cone_has_rmin(c);
  const int hasphi  = cone_has_phi(c);
  distz = fabs(p.z) - c->dz;
  done |= (distz > kConeTolerance && (p.z * d.z) >= 0.) || (fabs(distz) < kConeTolerance && (p.z * d.z) > 0.);
  if (done) return distance;
  outerRad = cone_radius(c, p.z, 0);
  rsq      = v3_perp2(p);
  done |= (rsq > minus_tol_sq(outerRad, c->outerTolerance)) && (v3_dot(d, cone_normal(c, p, 0)) >= 0.);
  if (done) return distance;
  distance = -1.0;
  inside   = distz < -kConeTolerance;
  inside &= rsq < minus_tol_sq(outerRad, c->outerTolerance);
  if (hasrmin) inside &= rsq > plus_tol_sq(cone_radius(c, p.z, 1), c->innerTolerance);
  if (hasphi) inside &= cone_in_sector(c, p.x, p.y, 0);
  done |= inside;
  if (done) return distance;
  distance = kInfLength;
  distz /= NonZero(fabs(d.z));
  hitx = p.x + distz * d.x;
  hity = p.y + distz * d.y;
  r2   = (hitx * hitx) + (hity * hity);
  top  = (p.z >= c->tolIz) && (r2 <= c->sqRmax2 + kTolerance);
  bot  = (p.z <= -c->tolIz) && (r2 <= c->sqRmax1 + kTolerance);
  okz  = top || bot;
  if (hasrmin) {
    top &= (r2 >= c->sqRmin2 - kTolerance);
    bot &= (r2 >= c->sqRmin1 - kTolerance);
    okz &= (top || bot);
  }
  if (hasphi) okz &= cone_in_sector(c, hitx, hity, 1);
  if (!done && okz) distance = distz;
  done |= okz;
  if (done) return distance;
  ok = cone_conical(c, p, d, 1, 0, &dr);
  ok &= dr < distance;
  if (!done && ok) distance = dr;
  done |= ok;
  if (done) return distance;
  if (hasrmin) {
    ok = cone_conical(c, p, d, 1, 1, &dr);
    ok &= dr < distance;
    if (!done && ok) distance = dr;
  }
  if (hasphi) { /* SectorType of UniversalCone is unknown: both planes, positive-direction check */
    double dist_phi;
    int ok_phi;
    cone_phi_plane(c, c->alongphi1x, c->alongphi1y, c->w.n1x, c->w.n1y, p, d, 1, 1, &dist_phi, &ok_phi);
    ok_phi &= dist_phi < distance;
    if (!done && ok_phi) distance = dist_phi;
    done |= ok_phi;
    cone_phi_plane(c, c->alongphi2x, c->alongphi2y, c->w.n2x, c->w.n2y, p, d, 1, 1, &dist_phi, &ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  return distance;
}

/* DistanceToOut (ConeImplementation.h:257-366), full phi */
static double cone_dist_out(const or_cone *c, v3 p, v3 d)
{
  int done = 0, outside, up, down, onz, ok;
  double distance = kInfLength, distz, rsq, outerRad, dirZInv, dr;
  const int hasrmin = cone_has_rmin(c);
  distz    = fabs(p.z) - c->dz;
  distance = -1.0;
  outside  = distz > kConeTolerance;
  rsq      = v3_perp2(p);
  outerRad = cone_radius(c, p.z, 0);
  outside |= rsq > plus_tol_sq(outerRad, c->outerTolerance);
  done |= outside;
  if (done) return distance;
  if (hasrmin && !outside) {
    outside |= rsq < minus_tol_sq(cone_radius(c, p.z, 1), c->innerTolerance);
    done |= outside;
    if (done) return distance;
  }
  done |= outside;
  if (done) return distance;
  up   = d.z > 0.;
  down = d.z < 0.;
  onz  = !outside && ((up && p.z > 0. && fabs(distz) < kConeTolerance) ||
                     (down && p.z < 0. && fabs(distz) < kConeTolerance));
  if (!done && onz) distance = distz;
  done |= onz;
  if (done) return distance;
  distance = kInfLength;
  dirZInv  = 1. / NonZero(d.z);
  if (up) distance = (c->dz - p.z) * dirZInv;
  if (down) distance = (-c->dz - p.z) * dirZInv;
  ok = cone_conical(c, p, d, 0, 0, &dr);
  if (!done && ok && dr < distance) distance = dr;
  if (hasrmin) {
    ok = cone_conical(c, p, d, 0, 1, &dr);
    if (!done && ok && dr < distance) distance = dr;
  }
  if (cone_has_phi(c)) {
    /* the outside test's phi part (ConeImplementation.h:293-297) only runs where the point is
     * already outside, so it never changes the result of the scalar kernel */
    double dist_phi;
    int ok_phi;
    const int onStart = wedge_on_surface(c->w.a1x, c->w.a1y, c->w.n1x, c->w.n1y, p); /* IsOnStartPhi */
    const int onEnd   = wedge_on_surface(c->w.a2x, c->w.a2y, c->w.n2x, c->w.n2y, p); /* IsOnEndPhi */
    const int cond    = (onStart && (d.x * -c->w.n1x + d.y * -c->w.n1y + d.z * -0.) > 0.) ||
                     (onEnd && (d.x * -c->w.n2x + d.y * -c->w.n2y + d.z * -0.) > 0.);
    if (!done && cond) distance = 0.;
    done |= cond;
    if (done) return distance;
    cone_phi_plane(c, c->alongphi1x, c->alongphi1y, c->w.n1x, c->w.n1y, p, d, 1, 0, &dist_phi, &ok_phi);
    ok_phi &= dist_phi < distance;
    if (!done && ok_phi) distance = dist_phi;
    done |= ok_phi;
    cone_phi_plane(c, c->alongphi2x, c->alongphi2y, c->w.n2x, c->w.n2y, p, d, 1, 0, &dist_phi, &ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  if (distance < 0. && fabs(distance) < kTolerance) distance = 0.;
  return distance;
}

/* SafeDistanceToConicalSurface (ConeImplementation.h:502-516) */
static inline double cone_safe_surface(const or_cone *c, v3 p, int inner)
{
  double rho = sqrt(v3_perp2(p));
  if (inner) {
    double pRMin = c->tanRMin * p.z + (c->rmin1 + c->rmin2) * 0.5;
    return (rho - pRMin) * c->invSecRMin;
  }
  {
    double pRMax = c->tanRMax * p.z + (c->rmax1 + c->rmax2) * 0.5;
    return (pRMax - rho) * c->invSecRMax;
  }
}

/* SafetyToIn (ConeImplementation.h:368-432), full phi */
static double cone_safe_in(const or_cone *c, v3 p)
{
  int inside;
  double safety, distz, outerRad, rsq, safeZ, so, si = -kInfLength;
  const int hasrmin = cone_has_rmin(c);
  distz    = fabs(p.z) - c->dz;
  safety   = -1.0;
  inside   = distz < -kConeTolerance;
  outerRad = cone_radius(c, p.z, 0);
  rsq      = v3_perp2(p);
  inside &= rsq < minus_tol_sq(outerRad, c->outerTolerance);
  if (hasrmin) inside &= rsq > plus_tol_sq(cone_radius(c, p.z, 1), c->innerTolerance);
  if (cone_has_phi(c) && inside) inside &= cone_in_sector(c, p.x, p.y, 0);
  if (inside) return safety;
  safeZ = fabs(p.z) - c->dz;
  so    = -cone_safe_surface(c, p, 0);
  if (hasrmin) si = -cone_safe_surface(c, p, 1);
  safety = or_max(safeZ, or_max(so, si));
  if (cone_has_phi(c)) safety = or_max(wedge_safe_in(&c->w, p), safety);
  if (fabs(safety) < kTolerance) safety = 0.;
  return safety;
}

/* SafetyToOut (ConeImplementation.h:434-499), full phi */
static double cone_safe_out(const or_cone *c, v3 p)
{
  int outside;
  double safety, distz, rsq, outerRad, safeZ, so, si = kInfLength;
  const int hasrmin = cone_has_rmin(c);
  distz    = fabs(p.z) - c->dz;
  rsq      = v3_perp2(p);
  safety   = -1.0;
  outside  = distz > kConeTolerance;
  outerRad = cone_radius(c, p.z, 0);
  outside |= rsq > plus_tol_sq(outerRad, c->outerTolerance);
  if (hasrmin) outside |= rsq < minus_tol_sq(cone_radius(c, p.z, 1), c->innerTolerance);
  if (outside) return safety;
  safeZ = c->dz - fabs(p.z);
  so    = cone_safe_surface(c, p, 0);
  if (hasrmin) si = cone_safe_surface(c, p, 1);
  safety = or_min(safeZ, or_min(so, si));
  if (cone_has_phi(c)) safety = or_min(wedge_safe_out(&c->w, p), safety);
  if (fabs(safety) < kTolerance) safety = 0.;
  return safety;
}

/* ConeHelpers<double>::GenericKernelForContainsAndInside (ConeUtilities.h:764-813) */
static void cone_generic_ci(const or_cone *c, v3 p, int forinside, int *cin, int *cout)
{
  double absz = fabs(p.z), r2, rmax;
  *cout = absz > (forinside ? c->dz + kConeTolerance : c->dz);
  if (forinside) *cin = absz < c->dz - kConeTolerance;
  if (*cout) return;
  r2   = p.x * p.x + p.y * p.y;
  rmax = (c->originalRmax1 == c->originalRmax2) ? c->originalRmax1 : c->outerSlope * p.z + c->outerOffset;
  *cout |= r2 > (forinside ? plus_tol_sq(rmax, c->outerTolerance) : rmax * rmax);
  if (forinside) *cin &= r2 < minus_tol_sq(rmax, c->outerTolerance);
  if (*cout) return;
  if (cone_has_rmin(c)) {
    double rmin = c->innerSlope * p.z + c->innerOffset;
    *cout |= r2 <= (forinside ? minus_tol_sq(rmin, c->innerTolerance) : rmin * rmin);
    if (forinside) *cin &= r2 > plus_tol_sq(rmin, c->innerTolerance);
    if (*cout) return;
  }
  if (cone_has_phi(c)) {
    int cinphi = 0, coutphi = 0;
    wedge_ci(&c->w, p, forinside, &cinphi, &coutphi);
    *cout |= coutphi;
    if (forinside) *cin &= cinphi;
  }
}

static int cone_contains(const or_cone *c, v3 p)
{
  int cin = 0, cout = 0;
  cone_generic_ci(c, p, 0, &cin, &cout);
  return !cout;
}

static int cone_inside(const or_cone *c, v3 p)
{
  int cin = 0, cout = 0, r = kSurfaceE;
  cone_generic_ci(c, p, 1, &cin, &cout);
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

/* UnplacedCone::Extent (source/UnplacedCone.cpp:146-206, the phi-aware definition compiled in) */
static void cone_extent(const or_cone *c, v3 *mn, v3 *mx)
{
  double max = c->o_rmax1 > c->o_rmax2 ? c->o_rmax1 : c->o_rmax2;
  double min = c->o_rmin1 > c->o_rmin2 ? c->o_rmin2 : c->o_rmin1;
  double Rin, Cx, Dx, Cy, Dy, Ax, Bx, Ay, By, temp;
  int phi0out, phi90out, phi180out, phi270out;
  *mn = v3_make(-max, -max, -c->dz);
  *mx = v3_make(max, max, c->dz);
  if (c->dphi == kTwoPi) return;
  Rin       = 0.5 * (max + min);
  phi0out   = !wedge_contains(&c->w, v3_make(Rin, 0, 0));
  phi90out  = !wedge_contains(&c->w, v3_make(0, Rin, 0));
  phi180out = !wedge_contains(&c->w, v3_make(-Rin, 0, 0));
  phi270out = !wedge_contains(&c->w, v3_make(0, -Rin, 0));
  if (!(phi0out || phi90out || phi180out || phi270out)) return;
  Cx = max * cos(c->sphi);
  Dx = max * cos(c->sphi + c->dphi);
  Cy = max * sin(c->sphi);
  Dy = max * sin(c->sphi + c->dphi);
  if (phi0out) mx->x = or_max(Cx, Dx);
  if (phi90out) mx->y = or_max(Cy, Dy);
  if (phi180out) mn->x = or_min(Cx, Dx);
  if (phi270out) mn->y = or_min(Cy, Dy);
  if (c->dphi >= kPi) return;
  Ax = min * cos(c->sphi);
  Bx = min * cos(c->sphi + c->dphi);
  Ay = min * sin(c->sphi);
  By = min * sin(c->sphi + c->dphi);
  temp  = or_max(Ax, Bx);
  mx->x = temp > mx->x ? temp : mx->x;
  temp  = or_max(Ay, By);
  mx->y = temp > mx->y ? temp : mx->y;
  temp  = or_min(Ax, Bx);
  mn->x = temp < mn->x ? temp : mn->x;
  temp  = or_min(Ay, By);
  mn->y = temp < mn->y ? temp : mn->y;
}

/* ================================================================== */
/* Trd (UniversalTrd): kernel/TrdImplementation.h                     */
/* ================================================================== */

/* TrdStruct(x1, x2, y1, y2, z) + CalculateCached (TrdStruct.h:65-70, 103-119).
 * fToleranceY is computed from the x half-lengths, as in the reference. */
static int trd_init(or_trd *t, const double *a, char *err, int errlen)
{
  if (!(a[0] >= 0 && a[1] >= 0 && a[2] >= 0 && a[3] >= 0 && a[4] > 0)) {
    set_err(err, errlen, "Trd: half-lengths must be >= 0 and dz > 0");
    return -1;
  }
  t->dx1 = a[0];
  t->dx2 = a[1];
  t->dy1 = a[2];
  t->dy2 = a[3];
  t->dz  = a[4];
  t->x2minusx1    = t->dx2 - t->dx1;
  t->y2minusy1    = t->dy2 - t->dy1;
  t->halfx1plusx2 = 0.5 * (t->dx1 + t->dx2);
  t->halfy1plusy2 = 0.5 * (t->dy1 + t->dy2);
  t->fx           = 0.5 * (t->dx1 - t->dx2) / t->dz;
  t->fy           = 0.5 * (t->dy1 - t->dy2) / t->dz;
  t->secxz        = sqrt(1 + t->fx * t->fx);
  t->secyz        = sqrt(1 + t->fy * t->fy);
  t->calfx        = 1. / sqrt(1.0 + t->fx * t->fx);
  t->calfy        = 1. / sqrt(1.0 + t->fy * t->fy);
  t->tolx         = kTolerance * sqrt(t->x2minusx1 * t->x2minusx1 + 4 * t->dz * t->dz);
  t->toly         = kTolerance * sqrt(t->x2minusx1 * t->x2minusx1 + 4 * t->dz * t->dz);
  return 0;
}

/* TrdTypes::checkVaryingY for UniversalTrd (TrdTypes.h:66-75) */
static inline int trd_varying_y(const or_trd *t) { return t->dy1 != t->dy2; }

/* TrdUtilities::FaceTrajectoryIntersection (TrdImplementation.h:80-138); *dist is
 * only written when the direction faces the plane (the reference's early return). */
static int trd_face(const or_trd *t, v3 pos, v3 dir, int forY, int mirrored, int toInside, double *dist)
{
  double alongV, posV, dirV, posK, dirK, fV, fK, halfKplus, v1, ndotv;
  if (forY) {
    alongV = t->y2minusy1; v1 = t->dy1; posV = pos.y; posK = pos.x; dirV = dir.y; dirK = dir.x;
    fK = t->fx; fV = t->fy; halfKplus = t->halfx1plusx2;
  } else {
    alongV = t->x2minusx1; v1 = t->dx1; posV = pos.x; posK = pos.y; dirV = dir.x; dirK = dir.y;
    fK = t->fy; fV = t->fx; halfKplus = t->halfy1plusy2;
  }
  if (mirrored) {
    posV *= -1.;
    dirV *= -1.;
  }
  ndotv  = dirV + fV * dir.z;
  int ok = toInside ? ndotv < 0. : ndotv > 0.;
  if (!ok) return 0;
  double alongZ = 2.0 * t->dz;
  *dist = (alongZ * (posV - v1) - alongV * (pos.z + t->dz)) / (dir.z * alongV - dirV * alongZ + kTiny);
  ok    = ok && *dist > (0. - kHalfTolerance);
  if (ok) {
    double hitz = pos.z + *dist * dir.z;
    ok          = ok && fabs(hitz) <= t->dz;
    double hitk = posK + *dist * dirK;
    double dK   = halfKplus - fK * hitz;
    ok          = ok && fabs(hitk) <= dK;
    if (ok && fabs(*dist) < kHalfTolerance) *dist = 0.0;
  }
  return ok;
}

/* TrdUtilities::Safety (TrdImplementation.h:140-168) */
static double trd_safety(const or_trd *t, v3 p, int inside)
{
  double safz = t->dz - fabs(p.z);
  double dist = safz;
  double distx = t->halfx1plusx2 - t->fx * p.z;
  int okx      = distx >= 0;
  double safx  = (distx - fabs(p.x)) * t->calfx;
  if (okx && safx < dist) dist = safx;
  if (trd_varying_y(t)) {
    double disty = t->halfy1plusy2 - t->fy * p.z;
    int oky      = disty >= 0;
    double safy  = (disty - fabs(p.y)) * t->calfy;
    if (oky && safy < dist) dist = safy;
  } else {
    double safy = t->dy1 - fabs(p.y);
    if (safy < dist) dist = safy;
  }
  if (!inside) dist = -dist;
  return dist;
}

/* TrdUtilities::UnplacedInside (TrdImplementation.h:170-214); UniversalTrd takes
 * the general cross-product test for y (HasVaryingY is kUnknown). */
static void trd_unplaced_inside(const or_trd *t, v3 p, int surfaceT, int *cin, int *cout)
{
  double pzPlusDz = p.z + t->dz;
  *cout = fabs(p.z) > (surfaceT ? t->dz + kHalfTolerance : t->dz);
  if (surfaceT) *cin = fabs(p.z) < t->dz - kHalfTolerance;
  /* PointLineOrientation: cross = vx * py - vy * px */
  double cross = t->x2minusx1 * pzPlusDz - (2.0 * t->dz) * (fabs(p.x) - t->dx1);
  if (surfaceT) {
    *cout = *cout || cross < -t->tolx;
    *cin  = *cin && cross > t->tolx;
  } else {
    *cout = *cout || cross < 0;
  }
  cross = t->y2minusy1 * pzPlusDz - (2.0 * t->dz) * (fabs(p.y) - t->dy1);
  if (surfaceT) {
    *cout = *cout || cross < -t->toly;
    *cin  = *cin && cross > t->toly;
  } else {
    *cout = *cout || cross < 0;
  }
}

static int trd_contains(const or_trd *t, v3 p) /* TrdImplementation.h:263-272 */
{
  int cin = 0, cout = 0;
  trd_unplaced_inside(t, p, 0, &cin, &cout);
  return !cout;
}

static int trd_inside(const or_trd *t, v3 p) /* TrdImplementation.h:274-298 */
{
  int cin = 0, cout = 0, r = kSurfaceE;
  trd_unplaced_inside(t, p, 1, &cin, &cout);
  if (cin) r = kInsideE;
  if (cout) r = kOutsideE;
  return r;
}

static inline double trd_clamp(double d) { return fabs(d) < kHalfTolerance ? 0.0 : d; }

/* TrdImplementation::DistanceToIn (TrdImplementation.h:300-394) */
static double trd_dist_in(const or_trd *t, v3 p, v3 d)
{
  double distance = kInfLength;
  int inz         = fabs(p.z) < t->dz - kHalfTolerance;
  double distx    = t->halfx1plusx2 - t->fx * p.z;
  int inx         = (distx - fabs(p.x)) * t->calfx > 0. + kHalfTolerance;
  double disty;
  int iny;
  const int vary = trd_varying_y(t);
  if (vary) {
    disty = t->halfy1plusy2 - t->fy * p.z;
    iny   = (disty - fabs(p.y)) * t->calfy > 0. + kHalfTolerance;
  } else {
    disty = fabs(p.y) - t->dy1;
    iny   = disty < 0. - kHalfTolerance;
  }
  int inside = inx && iny && inz;
  if (inside) distance = -1.;
  int done = inside;
  int okz  = p.z * d.z < 0.;
  okz      = okz && !inz;
  if (okz) {
    double distz = (fabs(p.z) - t->dz) / fabs(d.z);
    double hitx  = fabs(p.x + distz * d.x);
    double hity  = fabs(p.y + distz * d.y);
    int okzt     = p.z > (t->dz - kHalfTolerance) && hitx <= t->dx2 && hity <= t->dy2;
    int okzb     = p.z < (-t->dz + kHalfTolerance) && hitx <= t->dx1 && hity <= t->dy1;
    okz          = okz && (okzt || okzb);
    if (okz) distance = distz;
  }
  done = done || okz;
  if (done) return trd_clamp(distance);

  int okx = 0;
  if (!inx) {
    okx = trd_face(t, p, d, 0, 0, 1, &distx);
    if (okx) distance = distx;
    okx = trd_face(t, p, d, 0, 1, 1, &distx);
    if (okx) distance = distx;
  }
  done = done || okx;
  if (done) return trd_clamp(distance);

  if (vary) {
    if (!iny) {
      int oky = trd_face(t, p, d, 1, 0, 1, &disty);
      if (oky) distance = disty;
      oky = trd_face(t, p, d, 1, 1, 1, &disty);
      if (oky) distance = disty;
    }
  } else {
    if (!iny) {
      disty /= fabs(d.y);
      double zhit = p.z + disty * d.z;
      double xhit = p.x + disty * d.x;
      double dx   = t->halfx1plusx2 - t->fx * zhit;
      int oky     = p.y * d.y < 0 && disty > -kHalfTolerance && fabs(xhit) < dx && fabs(zhit) < t->dz;
      if (oky) distance = disty;
    }
  }
  return trd_clamp(distance);
}

/* TrdImplementation::DistanceToOut (TrdImplementation.h:396-499); the scalar
 * backend allows the early returns. */
static double trd_dist_out(const or_trd *t, v3 p, v3 d)
{
  double distance = 0.0;
  double invdir   = 1. / fabs(d.z + kTiny);
  double safz     = t->dz - fabs(p.z);
  int out         = safz < 0. - kHalfTolerance;
  double distx    = t->halfx1plusx2 - t->fx * p.z;
  out             = out || (distx - fabs(p.x)) * t->calfx < 0. - kHalfTolerance;
  double disty;
  const int vary = trd_varying_y(t);
  if (vary) {
    disty = t->halfy1plusy2 - t->fy * p.z;
    out   = out || (disty - fabs(p.y)) * t->calfy < 0. - kHalfTolerance;
  } else {
    disty = t->dy1 - fabs(p.y);
    out   = out || disty < 0. - kHalfTolerance;
  }
  if (out) return -1.;
  if (d.z > 0.) {
    double distz = (t->dz - p.z) * invdir;
    double hitx  = fabs(p.x + distz * d.x);
    double hity  = fabs(p.y + distz * d.y);
    if (hitx <= t->dx2 && hity <= t->dy2) return trd_clamp(distz);
  }
  if (d.z < 0.) {
    double distz = (p.z + t->dz) * invdir;
    double hitx  = fabs(p.x + distz * d.x);
    double hity  = fabs(p.y + distz * d.y);
    if (hitx <= t->dx1 && hity <= t->dy1) return trd_clamp(distz);
  }
  if (trd_face(t, p, d, 0, 0, 0, &distx)) return trd_clamp(distx);
  if (trd_face(t, p, d, 0, 1, 0, &distx)) return trd_clamp(distx);
  if (vary) {
    if (trd_face(t, p, d, 1, 0, 0, &disty)) return trd_clamp(disty);
    if (trd_face(t, p, d, 1, 1, 0, &disty)) distance = disty;
  } else {
    double plane = t->dy1;
    if (d.y < 0.) plane = -t->dy1;
    disty       = (plane - p.y) / d.y;
    double zhit = p.z + disty * d.z;
    double xhit = p.x + disty * d.x;
    double dx   = t->halfx1plusx2 - t->fx * zhit;
    int oky     = fabs(xhit) < dx && fabs(zhit) < t->dz;
    if (oky) distance = disty;
  }
  return trd_clamp(distance);
}

/* UnplacedTrd::Extent (UnplacedTrd.h:218-222) */
static void trd_extent(const or_trd *t, v3 *mn, v3 *mx)
{
  double mxx = t->dx1 > t->dx2 ? t->dx1 : t->dx2;
  double mxy = t->dy1 > t->dy2 ? t->dy1 : t->dy2;
  *mn        = v3_make(-mxx, -mxy, -t->dz);
  *mx        = v3_make(mxx, mxy, t->dz);
}

/* ================================================================== */
/* Trapezoid: kernel/TrapezoidImplementation.h with base/PlaneShell.h */
/* ================================================================== */

static inline v3 v3_cross(v3 a, v3 b) /* Vector3D::Cross (Vector3D.h:230-234) */
{
  return v3_make(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

static inline double v3_dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* UnplacedTrapezoid::MakeAPlane (source/UnplacedTrapezoid.cpp:568-619): the normal is
 * (p3 - p1) x (p4 - p2), normalised by multiplying with 1/Length(); d = -n.centroid. */
static void trap_make_plane(or_trap *t, v3 p1, v3 p2, v3 p3, v3 p4, int i)
{
  v3 n     = v3_cross(v3_sub(p3, p1), v3_sub(p4, p2));
  double r = 1. / sqrt(v3_dot3(n, n));
  n        = v3_make(n.x * r, n.y * r, n.z * r);
  v3 sum   = v3_add(v3_add(v3_add(p1, p2), p3), p4);
  v3 centr = v3_make(0.25 * sum.x, 0.25 * sum.y, 0.25 * sum.z);
  t->a[i]  = n.x;
  t->b[i]  = n.y;
  t->c[i]  = n.z;
  t->d[i]  = -v3_dot3(n, centr);
}

/* UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, Alpha1, dy2, dx3, dx4, Alpha2)
 * (UnplacedTrapezoid.h:56-64): tangents of the alphas, TrapezoidStruct::CalculateCached
 * (TrapezoidStruct.h:90-95), FromParametersToCorners + MakePlanes
 * (source/UnplacedTrapezoid.cpp:447-466, 630-675). */
static int trap_init(or_trap *t, const double *a, char *err, int errlen)
{
  if (!(a[0] > 0 && a[3] > 0 && a[7] > 0 && a[4] >= 0 && a[5] >= 0 && a[8] >= 0 && a[9] >= 0 &&
        fabs(a[1]) < 0.5 * kPi)) {
    set_err(err, errlen, "Trapezoid: needs dz, dy1, dy2 > 0, dx >= 0 and |theta| < pi/2");
    return -1;
  }
  t->dz = a[0]; t->theta = a[1]; t->phi = a[2]; t->dy1 = a[3]; t->dx1 = a[4]; t->dx2 = a[5];
  t->tanAlpha1 = tan(a[6]);
  t->dy2 = a[7]; t->dx3 = a[8]; t->dx4 = a[9];
  t->tanAlpha2  = tan(a[10]);
  t->tthetaCphi = tan(t->theta) * cos(t->phi);
  t->tthetaSphi = tan(t->theta) * sin(t->phi);
  double dxdyDy1 = t->tanAlpha1 * t->dy1;
  double dxdyDy2 = t->tanAlpha2 * t->dy2;
  double dxdzDz  = t->tthetaCphi * t->dz;
  double dydzDz  = t->tthetaSphi * t->dz;
  v3 pt[8];
  pt[0] = v3_make(-dxdzDz - dxdyDy1 - t->dx1, -dydzDz - t->dy1, -t->dz);
  pt[1] = v3_make(-dxdzDz - dxdyDy1 + t->dx1, -dydzDz - t->dy1, -t->dz);
  pt[2] = v3_make(-dxdzDz + dxdyDy1 - t->dx2, -dydzDz + t->dy1, -t->dz);
  pt[3] = v3_make(-dxdzDz + dxdyDy1 + t->dx2, -dydzDz + t->dy1, -t->dz);
  pt[4] = v3_make(+dxdzDz - dxdyDy2 - t->dx3, +dydzDz - t->dy2, +t->dz);
  pt[5] = v3_make(+dxdzDz - dxdyDy2 + t->dx3, +dydzDz - t->dy2, +t->dz);
  pt[6] = v3_make(+dxdzDz + dxdyDy2 - t->dx4, +dydzDz + t->dy2, +t->dz);
  pt[7] = v3_make(+dxdzDz + dxdyDy2 + t->dx4, +dydzDz + t->dy2, +t->dz);
  trap_make_plane(t, pt[0], pt[1], pt[5], pt[4], 0); /* ~ -Y */
  trap_make_plane(t, pt[2], pt[6], pt[7], pt[3], 1); /* ~ +Y */
  trap_make_plane(t, pt[0], pt[4], pt[6], pt[2], 2); /* ~ -X */
  trap_make_plane(t, pt[1], pt[3], pt[7], pt[5], 3); /* ~ +X */
  return 0;
}

static inline double trap_pdist(const or_trap *t, int i, v3 p)
{
  return t->a[i] * p.x + t->b[i] * p.y + t->c[i] * p.z + t->d[i];
}

static inline double trap_proj(const or_trap *t, int i, v3 d) { return t->a[i] * d.x + t->b[i] * d.y + t->c[i] * d.z; }

/* GenericKernelForContainsAndInside (TrapezoidImplementation.h:124-162, PlaneShell.h:130-151) */
static void trap_generic_ci(const or_trap *t, v3 p, int forInside, int *cin, int *cout)
{
  *cout = fabs(p.z) > (forInside ? t->dz + kHalfTolerance : t->dz);
  if (forInside) *cin = fabs(p.z) < t->dz - kHalfTolerance;
  for (int i = 0; i < 4; ++i) {
    double dist = trap_pdist(t, i, p);
    *cout       = *cout || dist > (forInside ? 0. + kHalfTolerance : 0.);
    if (forInside) *cin = *cin && dist < 0. - kHalfTolerance;
  }
}

static int trap_contains(const or_trap *t, v3 p)
{
  int cin = 0, cout = 0;
  trap_generic_ci(t, p, 0, &cin, &cout);
  return !cout;
}

static int trap_inside(const or_trap *t, v3 p) /* TrapezoidImplementation.h:107-122 */
{
  int cin = 0, cout = 0, r = kSurfaceE;
  trap_generic_ci(t, p, 1, &cin, &cout);
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

/* DistanceToIn (TrapezoidImplementation.h:177-216) with PlaneShell::DistanceToIn
 * (PlaneShell.h:161-213); the scalar backend takes every early return. */
static double trap_dist_in(const or_trap *t, v3 p, v3 d)
{
  double signZdir = or_sign(d.z);
  double max      = signZdir * t->dz - p.z;
  if (signZdir * max < 0.0 + kHalfTolerance) return kInfLength;
  double invdir = 1.0 / NonZero(d.z);
  double smax   = max * invdir;
  double smin   = -(signZdir * t->dz + p.z) * invdir;
  double pdist[4], proj[4], vdist[4];
  for (int i = 0; i < 4; ++i) {
    pdist[i] = trap_pdist(t, i, p);
    proj[i]  = trap_proj(t, i, d);
    vdist[i] = -pdist[i] / NonZero(proj[i]);
  }
  for (int i = 0; i < 4; ++i) {
    if (pdist[i] > 0. + kHalfTolerance && proj[i] >= 0.) return kInfLength;
    if (pdist[i] > 0. - kHalfTolerance && proj[i] > 0.) return kInfLength;
  }
  for (int i = 0; i < 4; ++i) {
    int posPoint     = pdist[i] > 0. - kHalfTolerance;
    int posDir       = proj[i] > 0;
    int fromInside   = !posPoint && posDir;
    int fromOutside  = posPoint && !posDir;
    if (fromInside && vdist[i] < smin) return kInfLength;
    if (fromOutside && vdist[i] > smax) return kInfLength;
    if (fromOutside && vdist[i] > smin) smin = vdist[i];
    if (fromInside && vdist[i] < smax) smax = vdist[i];
  }
  return smin <= smax ? smin : kInfLength;
}

/* DistanceToOut (TrapezoidImplementation.h:270-299) with PlaneShell::DistanceToOut
 * (PlaneShell.h:219-257) */
static double trap_dist_out(const or_trap *t, v3 p, v3 d)
{
  if (fabs(p.z) > t->dz + kHalfTolerance) return -1.0;
  double distance = kInfLength;
  double distz    = (or_sign(d.z) * t->dz - p.z) / NonZero(d.z);
  if (d.z != 0.) distance = distz;
  double distOut = kInfLength;
  for (int i = 0; i < 4; ++i) {
    double pdist = trap_pdist(t, i, p);
    double proj  = trap_proj(t, i, d);
    double vdist = -pdist / NonZero(proj);
    if (pdist > kHalfTolerance) distOut = -1.;
    if (proj > 0. && vdist < distOut) distOut = vdist;
  }
  if (distOut < distance) distance = distOut;
  return distance;
}

/* SafetyToIn / SafetyToOut (TrapezoidImplementation.h:341-401, PlaneShell.h:260-305) */
static double trap_safe_in(const or_trap *t, v3 p)
{
  double safety = fabs(p.z) - t->dz;
  for (int i = 0; i < 4; ++i) {
    double dist = trap_pdist(t, i, p);
    if (dist > safety) safety = dist;
  }
  return safety;
}

static double trap_safe_out(const or_trap *t, v3 p)
{
  double safety = t->dz - fabs(p.z);
  for (int i = 0; i < 4; ++i) {
    double dist = -trap_pdist(t, i, p);
    if (dist < safety) safety = dist;
  }
  return safety;
}

/* UnplacedTrapezoid::Extent via fromPlanesToCorners (source/UnplacedTrapezoid.cpp:297-337, 467-494) */
static void trap_extent(const or_trap *t, v3 *mn, v3 *mx)
{
  const double dz = t->dz;
  const double *A = t->a, *B = t->b, *C = t->c, *D = t->d;
  double py[8], px[8];
  py[0] = py[1] = -(D[0] - dz * C[0]) / B[0];
  py[2] = py[3] = -(D[1] - dz * C[1]) / B[1];
  py[4] = py[5] = -(D[0] + dz * C[0]) / B[0];
  py[6] = py[7] = -(D[1] + dz * C[1]) / B[1];
  px[0] = ((B[2] / B[0]) * (D[0] - dz * C[0]) - (D[2] - dz * C[2])) / A[2];
  px[1] = ((B[3] / B[0]) * (D[0] - dz * C[0]) - (D[3] - dz * C[3])) / A[3];
  px[2] = ((B[2] / B[1]) * (D[1] - dz * C[1]) - (D[2] - dz * C[2])) / A[2];
  px[3] = ((B[3] / B[1]) * (D[1] - dz * C[1]) - (D[3] - dz * C[3])) / A[3];
  px[4] = ((B[2] / B[0]) * (D[0] + dz * C[0]) - (D[2] + dz * C[2])) / A[2];
  px[5] = ((B[3] / B[0]) * (D[0] + dz * C[0]) - (D[3] + dz * C[3])) / A[3];
  px[6] = ((B[2] / B[1]) * (D[1] + dz * C[1]) - (D[2] + dz * C[2])) / A[2];
  px[7] = ((B[3] / B[1]) * (D[1] + dz * C[1]) - (D[3] + dz * C[3])) / A[3];
  mx->x = or_max(or_max(or_max(px[0], px[1]), or_max(px[2], px[3])), or_max(or_max(px[4], px[5]), or_max(px[6], px[7])));
  mn->x = or_min(or_min(or_min(px[0], px[1]), or_min(px[2], px[3])), or_min(or_min(px[4], px[5]), or_min(px[6], px[7])));
  mx->y = or_max(or_max(or_max(py[0], py[1]), or_max(py[2], py[3])), or_max(or_max(py[4], py[5]), or_max(py[6], py[7])));
  mn->y = or_min(or_min(or_min(py[0], py[1]), or_min(py[2], py[3])), or_min(or_min(py[4], py[5]), or_min(py[6], py[7])));
  mn->z = -dz;
  mx->z = dz;
}

/* ================================================================== */
/* Sphere: kernel/SphereImplementation.h, SphereUtilities.h,          */
/* Wedge_Evolution.h, ThetaCone_Evolution.h                           */
/* ================================================================== */

/* ---- evolution::Wedge pieces only the sphere uses ---- */

/* Wedge::IsPointOnSurfaceAndMovingOut<start, movingOut> (Wedge_Evolution.h:233-246): on the
 * face and moving along / against its inward normal */
static int wedge_moving(const or_wedge *w, int start, int movingOut, v3 p, v3 d)
{
  double ax = start ? w->a1x : w->a2x, ay = start ? w->a1y : w->a2y;
  double nx = start ? w->n1x : w->n2x, ny = start ? w->n1y : w->n2y;
  if (!wedge_on_surface(ax, ay, nx, ny, p)) return 0;
  double dn = d.x * -nx + d.y * -ny; /* dir.Dot(-normal); the normal has z = 0 */
  return movingOut ? dn > 0.005 * kHalfTolerance : dn < 0.005 * kHalfTolerance;
}

/* Wedge::DistanceToIn / DistanceToOut (Wedge_Evolution.h:393-446): distances to the two
 * half-planes, kInfLength unless the ray approaches the plane from the chosen side */
static void wedge_dist(const or_wedge *w, v3 p, v3 d, int toIn, double *dist1, double *dist2)
{
  double comp1 = d.x * w->n1x + d.y * w->n1y;
  double comp2 = d.x * w->n2x + d.y * w->n2y;
  *dist1 = kInfLength;
  *dist2 = kInfLength;
  if (toIn ? comp1 > 0. : comp1 < 0.) {
    double tmp = -(p.x * w->n1x + p.y * w->n1y) / comp1;
    if (tmp > 0.) *dist1 = tmp;
  }
  if (toIn ? comp2 > 0. : comp2 < 0.) {
    double tmp = -(p.x * w->n2x + p.y * w->n2y) / comp2;
    if (tmp > 0.) *dist2 = tmp;
  }
}

/* ---- ThetaCone (ThetaCone_Evolution.h) ---- */
#define kThHalfTol (0.5 * kTolerance) /* halfAngTolerance; kAngTolerance = kTolerance */
#define kThTolAng (2 * kTolerance * 10.)

/* ThetaCone(sTheta, dTheta) (ThetaCone_Evolution.h:62-82) */
static void theta_init(or_theta *c, double sT, double dT)
{
  c->sT = sT;
  c->dT = dT;
  c->eT = c->sT + c->dT;
  double ts = c->sT, te = c->eT;
  if (c->sT > kPi / 2) ts = kPi - c->sT;
  if (c->eT > kPi / 2) te = kPi - c->eT;
  c->tanS   = tan(ts);
  c->tanS2  = c->tanS * c->tanS;
  c->tanE   = tan(te);
  c->tanE2  = c->tanE * c->tanE;
  c->tanBis = tan(ts + (c->dT / 2));
  if (c->sT > kPi / 2 && c->eT > kPi / 2) c->tanBis = tan(ts - (c->dT / 2));
  c->slope1 = tan(kPi / 2 - c->sT);
  c->slope2 = tan(kPi / 2 - c->eT);
}

/* ThetaCone::IsCompletelyInside (ThetaCone_Evolution.h:655-730) */
static int theta_completely_inside(const or_theta *c, v3 p)
{
  const double sT = c->sT, eT = c->eT;
  double rho         = sqrt(v3_dot(p, p) - (p.z * p.z));
  double cone1Radius = fabs(p.z * c->tanS);
  double cone2Radius = fabs(p.z * c->tanE);
  int onZ  = p.z != 0. && p.x == 0. && p.y == 0.;
  int onXY = p.z == 0. && (p.x != 0. || p.y != 0.);
  int ci   = onZ && ((sT == 0. && eT == kPi) || (p.z > 0. && sT == 0.) || (p.z < 0. && eT == kPi));
  ci = ci || (!ci && (onXY && (sT < kHalfPi && eT > kHalfPi && (kHalfPi - sT) > kTolerance &&
                               (eT - kHalfPi) > kTolerance)));
  if (sT < kHalfPi + kThHalfTol) {
    if (eT < kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin = cone1Radius + kThTolAng;
      double tolAngMax = cone2Radius - kThTolAng;
      ci = ci || (!ci && (((rho <= tolAngMax) && (rho >= tolAngMin) && (p.z > 0.) && (sT != 0.)) ||
                          ((rho <= tolAngMax) && (sT == 0.) && (p.z > 0.))));
    }
    if (eT > kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin = cone1Radius + kThTolAng;
      double tolAngMax = cone2Radius + kThTolAng;
      ci = ci || (!ci && (((rho >= tolAngMin) && (p.z > 0.)) || ((rho >= tolAngMax) && (p.z < 0.))));
    }
    if (eT >= kHalfPi - kThHalfTol && eT <= kHalfPi + kThHalfTol) ci = ci && !(fabs(p.z) < kThHalfTol);
  }
  if (eT > kHalfPi + kThHalfTol) {
    if (sT >= kHalfPi - kThHalfTol && sT <= kHalfPi + kThHalfTol) ci = ci && !(fabs(p.z) < kThHalfTol);
    if (sT > kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin = cone1Radius - kThTolAng;
      double tolAngMax = cone2Radius + kThTolAng;
      ci = ci || (!ci && (((rho <= tolAngMin) && (rho >= tolAngMax) && (p.z < 0.) && (eT != kPi)) ||
                          ((rho <= tolAngMin) && (p.z < 0.) && (eT == kPi))));
    }
  }
  return ci;
}

/* ThetaCone::IsCompletelyOutside (ThetaCone_Evolution.h:733-805) */
static int theta_completely_outside(const or_theta *c, v3 p)
{
  const double sT = c->sT, eT = c->eT;
  double diff        = p.x * p.x + p.y * p.y;
  double rho         = sqrt(diff);
  double cone1Radius = fabs(p.z * c->tanS);
  double cone2Radius = fabs(p.z * c->tanE);
  int onZ  = p.z != 0. && p.x == 0. && p.y == 0.;
  int onXY = p.z == 0. && (p.x != 0. || p.y != 0.);
  int co   = onZ && ((sT != 0. && eT != kPi) || (p.z > 0. && sT != 0.) || (p.z < 0. && eT != kPi));
  co = co || (!co && (onXY && (((sT < kHalfPi) && (eT < kHalfPi) && ((kHalfPi - sT) > kTolerance) &&
                                ((kHalfPi - eT) > kTolerance)) ||
                               ((sT > kHalfPi && eT > kHalfPi) && ((sT - kHalfPi) > kTolerance) &&
                                ((eT - kHalfPi) > kTolerance)))));
  if (sT < kHalfPi + kThHalfTol) {
    if (eT < kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin2 = cone1Radius - kThTolAng;
      double tolAngMax2 = cone2Radius + kThTolAng;
      co = co || (!co && ((rho < tolAngMin2) || (rho > tolAngMax2) || (p.z < 0.)));
    }
    if (eT > kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin2 = cone1Radius - kThTolAng;
      double tolAngMax2 = cone2Radius - kThTolAng;
      co = co || (!co && (((rho < tolAngMin2) && (p.z > 0.)) || ((rho < tolAngMax2) && (p.z < 0.))));
    }
    if (eT >= kHalfPi - kThHalfTol && eT <= kHalfPi + kThHalfTol) co = co && !(fabs(p.z) < kThHalfTol);
  }
  if (eT > kHalfPi + kThHalfTol) {
    if (sT >= kHalfPi - kThHalfTol && sT <= kHalfPi + kThHalfTol) co = co && !(fabs(p.z) < kThHalfTol);
    if (sT > kHalfPi + kThHalfTol && sT < eT) {
      double tolAngMin2 = cone1Radius + kThTolAng;
      double tolAngMax2 = cone2Radius - kThTolAng;
      co = co || (!co && ((rho < tolAngMax2) || (rho > tolAngMin2) || (p.z > 0.)));
    }
  }
  return co;
}

/* ThetaCone::Contains (ThetaCone_Evolution.h:231-240) */
static inline int theta_contains(const or_theta *c, v3 p) { return !theta_completely_outside(c, p); }

/* ThetaCone::IsPointOnSurfaceAndMovingOut<start, movingOut> (ThetaCone_Evolution.h:164-229):
 * on the cone face (IsOnSurfaceGeneric) and moving along / against GetNormal<start> */
static int theta_moving(const or_theta *c, int start, int movingOut, v3 p, v3 d)
{
  double rhs  = fabs((start ? c->tanS : c->tanE) * p.z);
  double rho2 = p.x * p.x + p.y * p.y;
  if (!(rho2 >= minus_tol_sq(rhs, kTolerance) && rho2 <= plus_tol_sq(rhs, kTolerance))) return 0;
  v3 n = v3_make(p.x, p.y, -(start ? c->tanS2 : c->tanE2) * p.z);
  if (start ? c->sT <= kHalfPi : !(c->eT <= kHalfPi)) n = v3_make(-n.x, -n.y, -n.z);
  double dn = v3_dot(d, n);
  return movingOut ? dn > 0. : dn < 0.;
}

/* ThetaCone::DistanceToLine (ThetaCone_Evolution.h:358-365) */
static inline double theta_dist_line(double slope, double x, double y)
{
  double dist = (y - slope * x) / sqrt(1. + slope * slope);
  return fabs(dist);
}

/* ThetaCone::SafetyToIn (ThetaCone_Evolution.h:276-316) */
static double theta_safe_in(const or_theta *c, v3 p)
{
  const double sT = c->sT, eT = c->eT;
  double pointRad  = sqrt(p.x * p.x + p.y * p.y);
  double sfTh1     = theta_dist_line(c->slope1, pointRad, p.z);
  double sfTh2     = theta_dist_line(c->slope2, pointRad, p.z);
  double safeTheta = or_min(sfTh1, sfTh2);
  if (theta_contains(c, p)) return 0.;
  if (sT < kPi / 2 + kThHalfTol) {
    if (eT < kPi / 2 + kThHalfTol && sT < eT && p.z < 0.) safeTheta = sfTh2;
    if (eT > kPi / 2 + kThHalfTol && sT < eT) {
      if (p.z > 0.) safeTheta = sfTh1;
      if (p.z < 0.) safeTheta = sfTh2;
    }
  }
  if (eT > kPi / 2 + kThHalfTol && sT > kPi / 2 + kThHalfTol && sT < eT && p.z > 0.) safeTheta = sfTh1;
  return safeTheta;
}

/* ThetaCone::SafetyToOut (ThetaCone_Evolution.h:318-356) */
static double theta_safe_out(const or_theta *c, v3 p)
{
  const double sT = c->sT, eT = c->eT;
  double pointRad    = sqrt(p.x * p.x + p.y * p.y);
  double bisectorRad = fabs(p.z * c->tanBis);
  int cond           = 0;
  double sfTh1       = theta_dist_line(c->slope1, pointRad, p.z);
  double sfTh2       = theta_dist_line(c->slope2, pointRad, p.z);
  if (sT < kPi / 2 + kThHalfTol) {
    if (eT < kPi / 2 + kThHalfTol && sT < eT) cond = (pointRad < bisectorRad) && (sT != 0.);
    if (eT > kPi / 2 + kThHalfTol && sT < eT) cond = sfTh1 < sfTh2;
  }
  if (eT > kPi / 2 + kThHalfTol && sT > kPi / 2 + kThHalfTol && sT < eT)
    cond = !((pointRad < bisectorRad) && (eT != kPi));
  return cond ? sfTh1 : sfTh2;
}

/* The root clean-up ThetaCone::DistanceToIn applies to each cone root: a root within
 * 3 kTolerance of zero becomes 0 and sets `done`; a negative root becomes kInfLength unless
 * `done` is already set (ThetaCone_Evolution.h:387-395) */
static inline double theta_in_root(double root, int *done)
{
  *done = *done || (fabs(root) < 3. * kTolerance);
  if (fabs(root) < 3. * kTolerance) root = 0.;
  if (!*done && root < 0.) root = kInfLength;
  return root;
}

/* ThetaCone::DistanceToIn (ThetaCone_Evolution.h:367-496); dist1/dist2 and int1/int2 come
 * in as kInfLength and false and are only overwritten by the branches that apply */
static void theta_dist_in(const or_theta *c, v3 p, v3 d, double *dist1, double *dist2, int *int1, int *int2)
{
  const double sT = c->sT, eT = c->eT;
  int done          = 0;
  double firstRoot  = kInfLength, secondRoot = kInfLength;
  double pDotV2d    = p.x * d.x + p.y * d.y;
  double rho2       = p.x * p.x + p.y * p.y;
  double dirRho2    = d.x * d.x + d.y * d.y;
  double b          = pDotV2d - p.z * d.z * c->tanS2;
  double a          = dirRho2 - d.z * d.z * c->tanS2;
  double cc         = rho2 - p.z * p.z * c->tanS2;
  double d2         = b * b - a * cc;
  double aInv       = 1. / NonZero(a);
  if (d2 > 0.) firstRoot = (-b + sqrt(fabs(d2))) * aInv;
  firstRoot = theta_in_root(firstRoot, &done);

  double b2    = pDotV2d - p.z * d.z * c->tanE2;
  double a2    = dirRho2 - d.z * d.z * c->tanE2;
  double c2    = rho2 - p.z * p.z * c->tanE2;
  double d22   = b2 * b2 - a2 * c2;
  double a2Inv = 1. / NonZero(a2);
  if (d22 > 0.) secondRoot = (-b2 - sqrt(fabs(d22))) * a2Inv;
  if (!done && fabs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
  done = done || (fabs(secondRoot) < 3. * kTolerance);
  if (!done && secondRoot < 0.) secondRoot = kInfLength;

  if (sT < kHalfPi + kThHalfTol) {
    if (eT < kHalfPi + kThHalfTol && sT < eT) {
      *dist1 = firstRoot;
      *dist2 = secondRoot;
      double z1 = (p.z + *dist1 * d.z), z2 = (p.z + *dist2 * d.z);
      *int1 = ((d2 > 0.) && (z1 > 0.));
      *int2 = ((d22 > 0.) && (z2 > 0.));
    }
    if (eT >= kHalfPi - kThHalfTol && eT <= kHalfPi + kThHalfTol) {
      if (d.z > 0.) *dist2 = -p.z / d.z;
      double z2 = (p.z + *dist2 * d.z);
      *int2 = ((*dist2 != kInfLength) && (fabs(z2) < kThHalfTol));
    }
    if (eT > kHalfPi + kThHalfTol && sT < eT) {
      *dist1 = firstRoot;
      if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
      done       = 0;
      secondRoot = theta_in_root(secondRoot, &done);
      *dist2     = secondRoot;
      double z1 = (p.z + *dist1 * d.z), z2 = (p.z + *dist2 * d.z);
      *int1 = ((d2 > 0) && (*dist1 != kInfLength) && (z1 > 0.));
      *int2 = ((d22 > 0) && (*dist2 != kInfLength) && (z2 < 0.));
    }
  }
  if (sT >= kHalfPi - kThHalfTol && eT > kHalfPi + kThHalfTol && sT < eT) {
    if (d2 > 0.) firstRoot = (-b - sqrt(fabs(d2))) * aInv;
    done      = 0;
    firstRoot = theta_in_root(firstRoot, &done);
    *dist1    = firstRoot;
    if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
    done       = 0;
    secondRoot = theta_in_root(secondRoot, &done);
    *dist2     = secondRoot;
    double z1 = (p.z + *dist1 * d.z), z2 = (p.z + *dist2 * d.z);
    *int1 = ((d2 > 0) && (*dist1 != kInfLength) && (z1 < 0.));
    *int2 = ((d22 > 0) && (*dist2 != kInfLength) && (z2 < 0.));
  }
  if (sT >= kHalfPi - kThHalfTol && sT <= kHalfPi + kThHalfTol) {
    if (d.z < 0.) *dist1 = -p.z / d.z;
    double z1 = (p.z + *dist1 * d.z);
    *int1 = ((*dist1 != kInfLength) && (fabs(z1) < kThHalfTol));
  }
}

/* ThetaCone::DistanceToOut (ThetaCone_Evolution.h:498-652), same conventions */
static void theta_dist_out(const or_theta *c, v3 p, v3 d, double *dist1, double *dist2, int *int1, int *int2)
{
  const double sT = c->sT, eT = c->eT;
  double inf       = kInfLength;
  double firstRoot = kInfLength, secondRoot = kInfLength;
  double pDotV2d   = p.x * d.x + p.y * d.y;
  double rho2      = p.x * p.x + p.y * p.y;
  double b         = pDotV2d - p.z * d.z * c->tanS2;
  double a         = d.x * d.x + d.y * d.y - d.z * d.z * c->tanS2;
  double cc        = rho2 - p.z * p.z * c->tanS2;
  double d2        = b * b - a * cc;
  if (d2 < 0. && fabs(d2) < kHalfTolerance) d2 = 0.;
  if ((d2 >= 0.) && b >= 0. && a != 0.) firstRoot = ((-b - sqrt(fabs(d2))) / NonZero(a));
  if ((d2 >= 0.) && b < 0.) firstRoot = ((cc) / NonZero(-b + sqrt(fabs(d2))));
  if (firstRoot < 0.) firstRoot = kInfLength;

  double b2  = p.x * d.x + p.y * d.y - p.z * d.z * c->tanE2;
  double a2  = d.x * d.x + d.y * d.y - d.z * d.z * c->tanE2;
  double c2  = p.x * p.x + p.y * p.y - p.z * p.z * c->tanE2;
  double d22 = (b2 * b2) - (a2 * c2);
  if (d22 < 0. && fabs(d22) < kHalfTolerance) d22 = 0.;
  if ((d22 >= 0.) && b2 >= 0.) secondRoot = ((c2) / NonZero(-b2 - sqrt(fabs(d22))));
  if ((d22 >= 0.) && b2 < 0. && a2 != 0.) secondRoot = ((-b2 + sqrt(fabs(d22))) / NonZero(a2));
  if (secondRoot < 0. && fabs(secondRoot) > kTolerance) secondRoot = kInfLength;
  if (fabs(secondRoot) < kTolerance) secondRoot = 0.;

  if (sT < kPi / 2 + kThHalfTol) {
    if (eT < kPi / 2 + kThHalfTol && sT < eT) {
      *dist1 = firstRoot;
      *dist2 = secondRoot;
      double z1 = (p.z + *dist1 * d.z), z2 = (p.z + *dist2 * d.z);
      *int1 = ((d2 > 0) && (*dist1 != kInfLength) && ((z1) > -kHalfTolerance));
      *int2 = ((d22 > 0) && (*dist2 != kInfLength) && ((z2) > -kHalfTolerance));
      double dirRho2 = d.x * d.x + d.y * d.y;
      double zs = kInfLength, ze = kInfLength;
      if (sT != 0.) zs = dirRho2 / c->tanS;
      if (eT != 0.) ze = dirRho2 / c->tanE;
      int cond = (p.x == 0. && p.y == 0. && p.z == 0. && d.z < zs && d.z < ze);
      if (cond) *dist1 = 0.;
      if (cond) *dist2 = 0.;
      *int1 = *int1 || cond;
      *int2 = *int2 || cond;
    }
    if (eT >= kPi / 2 - kThHalfTol && eT <= kPi / 2 + kThHalfTol) {
      *dist1 = firstRoot;
      *dist2 = inf;
      if (d.z < 0.) *dist2 = -1. * p.z / d.z;
      double z2 = (p.z + *dist2 * d.z), z1 = (p.z + *dist1 * d.z);
      *int2 = ((*dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && !(d.z == 0.));
      *int1 = ((d2 >= 0) && (*dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && !(d.z == 0.));
    }
    if (eT > kPi / 2 + kThHalfTol && sT < eT) {
      *dist1 = firstRoot;
      if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / NonZero(a2));
      if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / NonZero(-b2 + sqrt(fabs(d22))));
      if (secondRoot < 0.) secondRoot = kInfLength;
      *dist2 = secondRoot;
      double z1 = (p.z + *dist1 * d.z), z2 = (p.z + *dist2 * d.z);
      *int1 = ((d2 >= 0) && (*dist1 != kInfLength) && ((z1) > -kHalfTolerance));
      *int2 = ((d22 >= 0) && (*dist2 != kInfLength) && ((z2) < kHalfTolerance));
    }
  }
  if (eT > kPi / 2 + kThHalfTol && sT < eT) {
    secondRoot = kInfLength;
    if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / NonZero(a2));
    if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / NonZero(-b2 + sqrt(fabs(d22))));
    *dist2 = secondRoot;
    if (sT > kPi / 2 + kThHalfTol) {
      if ((d2 >= 0.) && b > 0.) firstRoot = ((cc) / NonZero(-b - sqrt(fabs(d2))));
      if ((d2 >= 0.) && b <= 0. && a != 0.) firstRoot = ((-b + sqrt(fabs(d2))) / NonZero(a));
      if (firstRoot < 0.) firstRoot = kInfLength;
      *dist1    = firstRoot;
      double z1 = (p.z + *dist1 * d.z);
      *int1     = ((d2 > 0) && (*dist1 != kInfLength) && ((z1) < kHalfTolerance));
      double z2 = (p.z + *dist2 * d.z);
      *int2     = ((d22 > 0) && (*dist2 != kInfLength) && ((z2) < kHalfTolerance));
      double dirRho2 = d.x * d.x + d.y * d.y;
      double zs = -kInfLength, ze = -kInfLength;
      if (c->tanS != 0.) zs = -dirRho2 / c->tanS;
      if (c->tanE != 0.) ze = -dirRho2 / c->tanE;
      int cond = (p.x == 0. && p.y == 0. && p.z == 0. && d.z > zs && d.z > ze);
      if (cond) *dist1 = 0.;
      if (cond) *dist2 = 0.;
      *int1 = *int1 || cond;
      *int2 = *int2 || cond;
    }
  }
  if (sT >= kPi / 2 - kThHalfTol && sT <= kPi / 2 + kThHalfTol) {
    *dist2 = secondRoot;
    *dist1 = kInfLength;
    if (d.z > 0.) *dist1 = -1. * p.z / NonZero(d.z);
    double z1 = (p.z + *dist1 * d.z);
    double z2 = (p.z + *dist2 * d.z);
    *int1 = ((*dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && (d.z != 0.));
    *int2 = ((d22 >= 0) && (*dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && (d.z != 0.));
  }
}

/* ---- the sphere ---- */

/* SphereStruct(rmin, rmax, sphi, dphi, stheta, dtheta) (SphereStruct.h:285-304):
 * CheckPhiAngles and CheckThetaAngles set the checked angles and the full-range flags;
 * the Wedge and the ThetaCone keep the raw constructor angles.  Arguments for which the
 * reference only reports an error (dphi <= 0, stheta outside [0, pi], dtheta <= 0) are
 * rejected. */
static int sphere_init(or_sphere *t, const double *a, char *err, int errlen)
{
  const double rmin = a[0], rmax = a[1], sphi = a[2], dphi = a[3], stheta = a[4], dtheta = a[5];
  if (!(rmin >= 0 && rmax > rmin) || !(dphi > 0) || !(stheta >= 0 && stheta <= kPi) || !(dtheta > 0)) {
    set_err(err, errlen, "Sphere: needs 0 <= rmin < rmax, dphi > 0, 0 <= stheta <= pi and dtheta > 0");
    return -1;
  }
  t->rmin = rmin;
  t->rmax = rmax;
  /* CheckDPhiAngle / CheckSPhiAngle (SphereStruct.h:129-176) */
  if (dphi >= 2 * kPi - kAngTolerance * 0.5) {
    t->dPhi    = 2 * kPi;
    t->sPhi    = 0;
    t->fullPhi = 1;
  } else {
    t->fullPhi = 0;
    t->dPhi    = dphi;
    if (sphi < 0)
      t->sPhi = 2 * kPi - fmod(fabs(sphi), 2 * kPi);
    else
      t->sPhi = fmod(sphi, 2 * kPi);
    if (t->sPhi + t->dPhi > 2 * kPi) t->sPhi -= 2 * kPi;
  }
  /* CheckThetaAngles (SphereStruct.h:87-126) */
  t->sTheta = stheta;
  if (dtheta + stheta >= kPi)
    t->dTheta = kPi - stheta;
  else
    t->dTheta = dtheta;
  t->fullTheta = !(t->dTheta - t->sTheta < kPi);
  t->full      = t->fullPhi && t->fullTheta;
  t->eTheta    = t->sTheta + t->dTheta;
  wedge_init(&t->w, dphi, sphi);
  theta_init(&t->tc, stheta, dtheta);
  return 0;
}

/* SphereUtilities::IsCompletelyInside / IsCompletelyOutside (SphereUtilities.h:110-141):
 * the wedge and the theta cone take part whatever the ranges */
static int sphere_completely_inside(const or_sphere *t, v3 p)
{
  double rad = sqrt(v3_dot(p, p));
  int inRad  = (rad < (t->rmax - kTolerance)) && (rad > (t->rmin + kTolerance));
  int cin = 0, cout = 0;
  wedge_ci(&t->w, p, 1, &cin, &cout);
  int inTheta = theta_completely_inside(&t->tc, p);
  return inRad && cin && inTheta;
}

static int sphere_completely_outside(const or_sphere *t, v3 p)
{
  double rad = sqrt(v3_dot(p, p));
  int outRad = (rad > (t->rmax + kTolerance)) || (rad < (t->rmin - kTolerance));
  int cin = 0, cout = 0;
  wedge_ci(&t->w, p, 1, &cin, &cout);
  int outTheta = theta_completely_outside(&t->tc, p);
  return outRad || cout || outTheta;
}

/* SphereUtilities::IsPointOnSurfaceAndMovingOut (SphereUtilities.h:143-195) */
static int sphere_on_surface_moving(const or_sphere *t, v3 p, v3 d, int movingOut)
{
  double mag2 = v3_dot(p, p);
  int onOuter = mag2 <= plus_tol_sq(t->rmax, kTolerance) && mag2 >= minus_tol_sq(t->rmax, kTolerance);
  double dp   = v3_dot(d, p);
  int outer   = onOuter && (movingOut ? dp > kSqrtTolerance : dp < -kSqrtTolerance);
  int inner   = 0;
  if (t->rmin != 0.) {
    int onInner = mag2 <= plus_tol_sq(t->rmin, kTolerance) && mag2 >= minus_tol_sq(t->rmin, kTolerance);
    double dmp  = d.x * -p.x + d.y * -p.y + d.z * -p.z;
    inner       = onInner && (movingOut ? dmp > kSqrtTolerance : dmp < -kSqrtTolerance);
  }
  int phiFace = 0, thetaFace = 0;
  if (t->dPhi < (kTwoPi - kHalfTolerance))
    phiFace = wedge_moving(&t->w, 1, movingOut, p, d) || wedge_moving(&t->w, 0, movingOut, p, d);
  if (t->dTheta < (kPi - kHalfTolerance))
    thetaFace = theta_moving(&t->tc, 1, movingOut, p, d) || theta_moving(&t->tc, 0, movingOut, p, d);
  int inShell = (mag2 >= t->rmin * t->rmin) && (mag2 <= t->rmax * t->rmax);
  return ((outer || inner) && wedge_contains(&t->w, p) && theta_contains(&t->tc, p)) ||
         (phiFace && inShell && theta_contains(&t->tc, p)) || (thetaFace && inShell && wedge_contains(&t->w, p));
}

/* SphereImplementation::GenericKernelForContainsAndInside<ForInside> (SphereImplementation.h:89-136) */
static void sphere_ci(const or_sphere *t, v3 p, int forInside, int *cin, int *cout)
{
  double rad2 = v3_dot(p, p);
  if (t->rmin != 0.) {
    *cin  = rad2 <= minus_tol_sq(t->rmax, kTolerance) && rad2 >= plus_tol_sq(t->rmin, kTolerance);
    *cout = rad2 >= plus_tol_sq(t->rmax, kTolerance) || rad2 <= minus_tol_sq(t->rmin, kTolerance);
  } else {
    *cin  = rad2 <= minus_tol_sq(t->rmax, kTolerance);
    *cout = rad2 >= plus_tol_sq(t->rmax, kTolerance);
  }
  if (!t->fullPhi) {
    int ci = 0, co = 0;
    wedge_ci(&t->w, p, forInside, &ci, &co);
    *cout = *cout || co;
    if (forInside) *cin = *cin && ci;
  }
  if (!t->fullTheta) {
    int ci = forInside ? theta_completely_inside(&t->tc, p) : 0;
    int co = theta_completely_outside(&t->tc, p);
    *cout  = *cout || co;
    if (forInside) *cin = *cin && ci;
  }
}

static int sphere_contains(const or_sphere *t, v3 p) /* SphereImplementation.h:62-70 */
{
  int cin = 0, cout = 0;
  sphere_ci(t, p, 0, &cin, &cout);
  return !cout;
}

static int sphere_inside(const or_sphere *t, v3 p) /* SphereImplementation.h:74-87 */
{
  int cin = 0, cout = 0, r = kSurfaceE;
  sphere_ci(t, p, 1, &cin, &cout);
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

/* SphereImplementation::GetMinDistFromPhi<DistToIn> (SphereImplementation.h:343-386): the
 * nearer, else the farther, phi-plane crossing that lies on its half-plane, strictly inside
 * the radial shell and within the theta range */
static void sphere_min_dist_phi(const or_sphere *t, v3 p, v3 d, int toIn, double *distance)
{
  double distPhi1 = kInfLength, distPhi2 = kInfLength;
  wedge_dist(&t->w, p, d, toIn, &distPhi1, &distPhi2);
  const or_wedge *w = &t->w;
  double dist = or_min(distPhi1, distPhi2);
  v3 tmp      = v3_add(p, v3_scale(dist, d));
  double rad2 = v3_dot(tmp, tmp);
  int onFace  = ((dist == distPhi1) && wedge_on_surface(w->a1x, w->a1y, w->n1x, w->n1y, tmp)) ||
               ((dist == distPhi2) && wedge_on_surface(w->a2x, w->a2y, w->n2x, w->n2y, tmp));
  int cond1 = onFace && (rad2 > t->rmin * t->rmin) && (rad2 < t->rmax * t->rmax) && theta_contains(&t->tc, tmp);
  if (cond1) *distance = or_min(dist, *distance);
  dist   = or_max(distPhi1, distPhi2);
  tmp    = v3_add(p, v3_scale(dist, d));
  rad2   = v3_dot(tmp, tmp);
  onFace = ((dist == distPhi1) && wedge_on_surface(w->a1x, w->a1y, w->n1x, w->n1y, tmp)) ||
           ((dist == distPhi2) && wedge_on_surface(w->a2x, w->a2y, w->n2x, w->n2y, tmp));
  int cond2 = onFace && (rad2 > t->rmin * t->rmin) && (rad2 < t->rmax * t->rmax) && theta_contains(&t->tc, tmp);
  if (!cond1 && cond2) *distance = or_min(dist, *distance);
}

/* DistanceToIn (SphereImplementation.h:138-256) */
static double sphere_dist_in(const or_sphere *t, v3 p, v3 d)
{
  double rad2    = v3_dot(p, p);
  double pDotV3d = v3_dot(p, d);
  double c       = rad2 - t->rmax * t->rmax;
  if (sphere_completely_inside(t, p)) return -1.0;
  if (sphere_on_surface_moving(t, p, d, 0)) return 0.0;
  double d2 = (pDotV3d * pDotV3d - c);
  if (d2 < 0. || ((c > 0.) && (pDotV3d > 0.))) return kInfLength;
  double sd1 = kInfLength, sd2 = kInfLength;
  if (d2 >= 0.) sd1 = (-pDotV3d - sqrt(fabs(d2)));
  double outerDist = kInfLength, innerDist = kInfLength;
  if (t->full) {
    if (sd1 >= 0.) outerDist = sd1;
  } else {
    v3 tmp = v3_add(p, v3_scale(sd1, d));
    if (wedge_contains(&t->w, tmp) && theta_contains(&t->tc, tmp) && (sd1 >= 0.)) outerDist = sd1;
  }
  if (t->rmin != 0.) {
    c  = rad2 - t->rmin * t->rmin;
    d2 = pDotV3d * pDotV3d - c;
    if (d2 >= 0.) sd2 = (-pDotV3d + sqrt(fabs(d2)));
    if (t->full) {
      if (sd2 >= 0.) innerDist = sd2;
    } else {
      v3 tmp = v3_add(p, v3_scale(sd2, d));
      if ((sd2 >= 0.) && wedge_contains(&t->w, tmp) && theta_contains(&t->tc, tmp)) innerDist = sd2;
    }
  }
  double distance = or_min(outerDist, innerDist);
  if (!t->fullPhi) sphere_min_dist_phi(t, p, d, 1, &distance);
  double distThetaMin = kInfLength;
  if (!t->fullTheta) {
    int int1 = 0, int2 = 0;
    double dt1 = kInfLength, dt2 = kInfLength;
    theta_dist_in(&t->tc, p, d, &dt1, &dt2, &int1, &int2);
    v3 c1 = v3_add(p, v3_scale(dt1, d)), c2 = v3_add(p, v3_scale(dt2, d));
    double r1 = v3_dot(c1, c1), r2 = v3_dot(c2, c2);
    int valid1 = (r1 >= t->rmin * t->rmin && r1 <= t->rmax * t->rmax) && int1;
    int valid2 = (r2 >= t->rmin * t->rmin && r2 <= t->rmax * t->rmax) && int2;
    if (!t->fullPhi) {
      valid1 = valid1 && wedge_contains(&t->w, c1);
      valid2 = valid2 && wedge_contains(&t->w, c2);
    }
    if (valid2 && !valid1) distThetaMin = dt2;
    if (valid1 && !valid2) distThetaMin = dt1;
    if (valid1 && valid2) distThetaMin = or_min(dt1, dt2);
  }
  distance = or_min(distThetaMin, distance);
  /* a ray aimed at the centre of a theta section enters at the apex */
  v3 toC        = v3_make(0. - p.x, 0. - p.y, 0. - p.z);
  double m2     = v3_dot(toC, toC);
  double newDist = sqrt(m2);
  double un     = sqrt(m2 + DBL_MIN);
  if ((t->sTheta > kHalfTolerance || t->eTheta < (kPi - kHalfTolerance)) && (fabs(toC.x / un - d.x) < kHalfTolerance) &&
      (fabs(toC.y / un - d.y) < kHalfTolerance) && (fabs(toC.z / un - d.z) < kHalfTolerance))
    distance = or_min(distance, newDist);
  return distance;
}

/* DistanceToOut (SphereImplementation.h:258-341) */
static double sphere_dist_out(const or_sphere *t, v3 p, v3 d)
{
  double pDotV3d = v3_dot(p, d);
  double rad2    = v3_dot(p, p);
  double c       = rad2 - t->rmax * t->rmax;
  if (sphere_completely_outside(t, p)) return -1.0;
  if (sphere_on_surface_moving(t, p, d, 1)) return 0.0;
  double sd1 = kInfLength, sd2 = kInfLength;
  double d2  = (pDotV3d * pDotV3d - c);
  if (d2 >= 0.) sd1 = (-pDotV3d + sqrt(fabs(d2)));
  if (t->rmin != 0.) {
    c  = rad2 - t->rmin * t->rmin;
    d2 = (pDotV3d * pDotV3d - c);
    if ((d2 >= 0.) && (pDotV3d < 0.)) sd2 = (-pDotV3d - sqrt(fabs(d2)));
  }
  double snxt  = or_min(sd1, sd2);
  int condSemi = ((t->sTheta == 0. && t->eTheta == kPi / 2.) && d.z >= 0.) ||
                 ((t->sTheta == kPi / 2. && t->eTheta == kPi) && d.z <= 0.);
  if (condSemi) return snxt;
  double distThetaMin = kInfLength;
  if (!t->fullTheta) {
    int int1 = 0, int2 = 0;
    double dt1 = kInfLength, dt2 = kInfLength;
    theta_dist_out(&t->tc, p, d, &dt1, &dt2, &int1, &int2);
    if (int2 && !int1) distThetaMin = dt2;
    if (!int2 && int1) distThetaMin = dt1;
    if (int2 && int1) distThetaMin = or_min(dt1, dt2);
  }
  double distance = or_min(distThetaMin, snxt);
  if (!t->fullPhi) {
    if (t->dPhi <= kPi) {
      double dp1, dp2;
      wedge_dist(&t->w, p, d, 0, &dp1, &dp2);
      distance = or_min(or_min(dp1, dp2), distance);
    } else {
      sphere_min_dist_phi(t, p, d, 0, &distance);
    }
  }
  return distance;
}

/* SafetyToIn / SafetyToOut (SphereImplementation.h:388-479) */
static double sphere_safe_in(const or_sphere *t, v3 p)
{
  double rad = sqrt(v3_dot(p, p));
  int cin = 0, cout = 0;
  sphere_ci(t, p, 1, &cin, &cout);
  if (cin) return -1.0;
  if (!cin && !cout) return 0.0;
  double safety;
  if (t->rmin != 0.) {
    double safeRMin = t->rmin - rad;
    double safeRMax = rad - t->rmax;
    safety          = safeRMin > safeRMax ? safeRMin : safeRMax;
  } else {
    safety = rad - t->rmax;
  }
  if (!t->fullPhi) safety = or_max(wedge_safe_in(&t->w, p), safety);
  if (!t->fullTheta) safety = or_max(theta_safe_in(&t->tc, p), safety);
  return safety;
}

static double sphere_safe_out(const or_sphere *t, v3 p)
{
  double rad = sqrt(v3_dot(p, p));
  int cin = 0, cout = 0;
  sphere_ci(t, p, 1, &cin, &cout);
  if (cout) return -1.0;
  if (!cin && !cout) return 0.0;
  double safety;
  if (t->rmin != 0.) {
    double safeRMin = (rad - t->rmin);
    double safeRMax = (t->rmax - rad);
    safety          = safeRMin < safeRMax ? safeRMin : safeRMax;
  } else {
    safety = t->rmax - rad;
  }
  if (!t->fullPhi) safety = or_min(wedge_safe_out(&t->w, p), safety);
  if (!t->fullTheta) safety = or_min(theta_safe_out(&t->tc, p), safety);
  return safety;
}

/* UnplacedSphere::Extent with the phi and theta cuts (source/UnplacedSphere.cpp:74-158) */
static void sphere_extent(const or_sphere *t, v3 *mn, v3 *mx)
{
  const double rmax = t->rmax, rmin = t->rmin;
  *mn = v3_make(-rmax, -rmax, -rmax);
  *mx = v3_make(rmax, rmax, rmax);
  double eTheta = t->sTheta + t->dTheta;
  if (t->full) return;
  double st1 = 0., st2 = 0.;
  if (!t->fullTheta) {
    mx->z = ((t->sTheta <= kPi / 2.) ? rmax : rmin) * cos(t->sTheta);
    mn->z = ((eTheta <= kPi / 2.) ? rmin : rmax) * cos(eTheta);
    st1   = sin(t->sTheta);
    st2   = sin(t->eTheta);
    if (t->sTheta <= kPi / 2.) {
      if ((eTheta) < kPi / 2.) {
        mx->x = rmax * st2;
        mn->x = -rmax * st2;
        mx->y = rmax * st2;
        mn->y = -rmax * st2;
      }
    } else {
      mx->x = rmax * st1;
      mn->x = -rmax * st1;
      mx->y = rmax * st1;
      mn->y = -rmax * st1;
    }
  }
  if (!t->fullPhi) {
    double Rmax = rmax;
    if (t->sTheta > kPi / 2.) Rmax *= st1;
    if (eTheta < kPi / 2.) Rmax *= st2;
    double Rmin = rmin * or_min(st1, st2);
    double Rin  = 0.5 * (Rmax + Rmin);
    int phi0out   = !wedge_contains(&t->w, v3_make(Rin, 0, 0));
    int phi90out  = !wedge_contains(&t->w, v3_make(0, Rin, 0));
    int phi180out = !wedge_contains(&t->w, v3_make(-Rin, 0, 0));
    int phi270out = !wedge_contains(&t->w, v3_make(0, -Rin, 0));
    if (!(phi0out || phi90out || phi180out || phi270out)) return;
    double Cx = Rmax * cos(t->sPhi), Dx = Rmax * cos(t->sPhi + t->dPhi);
    double Cy = Rmax * sin(t->sPhi), Dy = Rmax * sin(t->sPhi + t->dPhi);
    if (phi0out) mx->x = or_max(Cx, Dx);
    if (phi90out) mx->y = or_max(Cy, Dy);
    if (phi180out) mn->x = or_min(Cx, Dx);
    if (phi270out) mn->y = or_min(Cy, Dy);
    if (t->dPhi >= kPi) return;
    double Ax = Rmin * cos(t->sPhi), Bx = Rmin * cos(t->sPhi + t->dPhi);
    double Ay = Rmin * sin(t->sPhi), By = Rmin * sin(t->sPhi + t->dPhi);
    double temp;
    temp  = or_max(Ax, Bx);
    mx->x = temp > mx->x ? temp : mx->x;
    temp  = or_max(Ay, By);
    mx->y = temp > mx->y ? temp : mx->y;
    temp  = or_min(Ax, Bx);
    mn->x = temp < mn->x ? temp : mn->x;
    temp  = or_min(Ay, By);
    mn->y = temp < mn->y ? temp : mn->y;
  }
}

/* ================================================================== */
/* Polycone (full phi): kernel/PolyconeImplementation.h over the      */
/* ConeStruct sections of PolyconeStruct                               */
/* ================================================================== */

/* UnplacedPolycone(phistart, deltaphi, Nz, z, rmin, rmax) -> PolyconeStruct::Init
 * (UnplacedPolycone.h:78-88, PolyconeStruct.h:144-291): planes reversed when z runs
 * downwards, one section per z step larger than kTolerance, each section a ConeStruct
 * built with the raw phi arguments, shift = centre of the section in z.  The reference
 * only prints a message for rmin > rmax or a z direction change; both are rejected here. */
static int polycone_init(or_polycone *t, const double *a, char *err, int errlen)
{
  const double sphi = a[0], dphi = a[1];
  const int nz      = (int)a[2];
  const double *z0 = a + 3, *rin0 = a + 3 + nz, *rout0 = a + 3 + 2 * nz;
  double *z = (double *)malloc(sizeof(double) * (size_t)nz * 3), *rin = z + nz, *rout = z + 2 * nz;
  int i, rev = z0[0] > z0[nz - 1];
  if (!z) return -1;
  for (i = 0; i < nz; ++i) {
    z[i]    = rev ? z0[nz - 1 - i] : z0[i];
    rin[i]  = rev ? rin0[nz - 1 - i] : rin0[i];
    rout[i] = rev ? rout0[nz - 1 - i] : rout0[i];
  }
  /* SetAndCheckDPhiAngle, SetAndCheckSPhiAngle and the override that follows them
   * (PolyconeStruct.h:152-184, 355-390): the sections' cones take the raw angles */
  t->deltaPhi = dphi >= kTwoPi - 0.5 * kAngTolerance ? kTwoPi : dphi;
  t->startPhi = 0;
  if (dphi <= 0. || dphi > kTwoPi - kTolerance) {
    t->deltaPhi = kTwoPi;
  } else {
    t->startPhi = sphi;
    while (t->startPhi < 0) t->startPhi += kTwoPi;
  }
  for (i = 0; i < nz; ++i) {
    if (!(rin[i] >= 0 && rout[i] >= rin[i]) || (i > 0 && !(z[i] >= z[i - 1]))) {
      free(z);
      set_err(err, errlen, "Polycone: needs 0 <= rmin <= rmax and monotonic z planes");
      return -1;
    }
  }
  t->zs    = (double *)malloc(sizeof(double) * (size_t)nz);
  t->shift = (double *)malloc(sizeof(double) * (size_t)nz);
  t->sec   = (or_cone *)calloc((size_t)nz, sizeof(or_cone));
  t->nsec  = 0;
  if (!t->zs || !t->shift || !t->sec) {
    free(z);
    return -1;
  }
  double prevZ = z[0], prevRmax = 0, prevRmin = 0;
  int dirZ = 1, nzs = 0;
  if (z[1] < z[0]) dirZ = -1;
  for (i = 0; i < nz; ++i) {
    double rMin = rin[i], rMax = rout[i], zz = z[i];
    if (i > 0) {
      if (((zz > prevZ + kTolerance) && (dirZ > 0)) || ((zz < prevZ - kTolerance) && (dirZ < 0))) {
        double dz       = (zz - prevZ) / 2;
        double cpar[7]  = {prevRmin, prevRmax, rMin, rMax, dz, sphi, dphi};
        if (cone_init(&t->sec[t->nsec], cpar, err, errlen)) {
          free(z);
          return -1;
        }
        t->zs[nzs++]        = zz;
        t->shift[t->nsec++] = t->zs[nzs - 2] + 0.5 * (t->zs[nzs - 1] - t->zs[nzs - 2]);
      }
    } else {
      t->zs[nzs++] = zz;
    }
    prevZ    = zz;
    prevRmin = rMin;
    prevRmax = rMax;
  }
  free(z);
  if (t->nsec == 0) {
    set_err(err, errlen, "Polycone: no section longer than kTolerance");
    return -1;
  }
  return 0;
}

/* PolyconeStruct::GetSectionIndex (PolyconeStruct.h:302-311) */
static int polycone_section_index(const or_polycone *t, double zpos)
{
  if (zpos < t->zs[0]) return -1;
  for (int i = 0; i < t->nsec; ++i)
    if (zpos >= t->zs[i] && zpos <= t->zs[i + 1]) return i;
  return -2;
}

static inline v3 pcon_local(const or_polycone *t, int i, v3 p) { return v3_make(p.x, p.y, p.z - t->shift[i]); }

/* GenericKernelForASection (PolyconeImplementation.h:69-97) */
static void polycone_section_ci(const or_polycone *t, int isect, v3 p, int forInside, int *cin, int *cout)
{
  if (isect < 0) {
    *cin  = 0;
    *cout = 1;
    return;
  }
  cone_generic_ci(&t->sec[isect], pcon_local(t, isect, p), forInside, cin, cout);
}

/* GenericKernelForContainsAndInside (PolyconeImplementation.h:127-187); cin/cout keep
 * the caller's initial values where the reference leaves them untouched */
static void polycone_ci(const or_polycone *t, v3 p, int forInside, int *cin, int *cout)
{
  int indexLow  = polycone_section_index(t, p.z - kTolerance);
  int indexHigh = polycone_section_index(t, p.z + kTolerance);
  if (indexLow < 0 && indexHigh < 0) {
    *cout = 1;
    return;
  }
  if (indexLow < 0 && indexHigh == 0) {
    polycone_section_ci(t, 0, p, forInside, cin, cout);
    return;
  }
  if (indexHigh < 0 && indexLow == (t->nsec - 1)) {
    polycone_section_ci(t, t->nsec - 1, p, forInside, cin, cout);
    return;
  }
  if (indexLow >= 0 && indexHigh >= 0) {
    if (indexLow == indexHigh) {
      polycone_section_ci(t, indexLow, p, forInside, cin, cout);
      return;
    }
    int secInLow = 0, secOutLow = 0, secInHigh = 0, secOutHigh = 0;
    polycone_section_ci(t, indexLow, p, forInside, &secInLow, &secOutLow);
    polycone_section_ci(t, indexHigh, p, forInside, &secInHigh, &secOutHigh);
    int surfLow  = !secInLow && !secOutLow;
    int surfHigh = !secInHigh && !secOutHigh;
    if (surfLow && surfHigh) {
      *cin = 1;
      return;
    }
    if (secOutLow && secOutHigh) {
      *cout = 1;
      return;
    }
  }
}

static int polycone_contains(const or_polycone *t, v3 p) /* PolyconeImplementation.h:99-108 */
{
  int cin = 0, cout = 0;
  polycone_ci(t, p, 0, &cin, &cout);
  return !cout;
}

static int polycone_inside(const or_polycone *t, v3 p) /* PolyconeImplementation.h:112-125 */
{
  int cin = 0, cout = 0, r = kSurfaceE;
  polycone_ci(t, p, 1, &cin, &cout);
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

/* DistanceToIn (PolyconeImplementation.h:189-237): sections visited from the point's own
 * along the direction's z sign until one is hit */
static double polycone_dist_in(const or_polycone *t, v3 p, v3 v)
{
  double distance = kInfLength;
  int increment   = (v.z > 0) ? 1 : -1;
  if (fabs(v.z) < kTolerance) increment = 0;
  int index = polycone_section_index(t, p.z);
  if (index == -1) index = 0;
  if (index == -2) index = t->nsec - 1;
  do {
    distance = cone_dist_in(&t->sec[index], pcon_local(t, index, p), v);
    if (distance < kInfLength || !increment) break;
    index += increment;
  } while (index >= 0 && index < t->nsec);
  return distance;
}

/* DistanceToOut (PolyconeImplementation.h:239-379) */
static double polycone_dist_out(const or_polycone *t, v3 point, v3 dir)
{
  double distance = kInfLength;
  v3 pn           = point;
  if (t->nsec == 1) return cone_dist_out(&t->sec[0], pcon_local(t, 0, point), dir);
  int indexLow  = polycone_section_index(t, point.z - kTolerance);
  int indexHigh = polycone_section_index(t, point.z + kTolerance);
  int index     = 0;
  if (indexLow < 0 && indexHigh < 0) {
    return -1;
  } else if (indexLow < 0 && indexHigh >= 0) {
    index = indexHigh;
    if (cone_inside(&t->sec[index], pcon_local(t, index, point)) == kOutsideE) return -1;
  } else if (indexLow != indexHigh && (indexLow >= 0)) {
    if (cone_inside(&t->sec[indexLow], pcon_local(t, indexLow, point)) == kOutsideE)
      index = indexHigh;
    else
      index = indexLow;
  } else {
    index = indexLow;
    if (index < 0) index = polycone_section_index(t, point.z);
  }
  if (index < 0) {
    return 0.;
  } else {
    if (cone_inside(&t->sec[index], pcon_local(t, index, point)) == kOutsideE) return -1;
  }
  double totalDistance = 0., dist;
  int increment        = (dir.z > 0) ? 1 : -1;
  if (fabs(dir.z) < kTolerance) increment = 0;
  int istep = 0;
  do {
    if ((totalDistance != 0) || (istep < 2)) {
      pn = v3_make(point.x + totalDistance * dir.x, point.y + totalDistance * dir.y, point.z + totalDistance * dir.z);
      pn.z -= t->shift[index];
      if (cone_inside(&t->sec[index], pn) == kOutsideE) break;
    } else
      pn.z -= t->shift[index];
    istep++;
    dist = cone_dist_out(&t->sec[index], pn, dir);
    if (dist == -1) return distance;
    if (fabs(dist) < 0.5 * kTolerance) {
      int index1 = index;
      if ((index > 0) && (index < t->nsec - 1)) {
        index1 += increment;
      } else {
        if ((index == 0) && (increment > 0)) index1 += increment;
        if ((index == t->nsec - 1) && (increment < 0)) index1 += increment;
      }
      double td = totalDistance + dist;
      v3 pte    = v3_make(point.x + td * dir.x, point.y + td * dir.y, point.z + td * dir.z);
      pte.z -= t->shift[index1];
      if (cone_inside(&t->sec[index1], pte) == 3 || (increment == 0)) break;
    }
    totalDistance += dist;
    index += increment;
  } while (increment != 0 && index >= 0 && index < t->nsec);
  return totalDistance;
}

/* SafetyToIn (PolyconeImplementation.h:381-450) */
static double polycone_safe_in(const or_polycone *t, v3 p)
{
  int index = polycone_section_index(t, p.z);
  int needZ = 0;
  double safety, minSafety;
  if (index < 0) {
    needZ = 1;
    if (index == -1) index = 0;
    if (index == -2) index = t->nsec - 1;
  }
  safety = cone_safe_in(&t->sec[index], pcon_local(t, index, p));
  if (needZ) return safety;
  if (safety < kTolerance) return safety;
  minSafety    = safety;
  double zbase = t->zs[index + 1];
  for (int i = index + 1; i < t->nsec; ++i) {
    double dz = t->zs[i] - zbase;
    if (dz >= minSafety) break;
    safety = cone_safe_in(&t->sec[i], pcon_local(t, i, p));
    if (safety < minSafety) minSafety = safety;
  }
  if (index > 0) {
    zbase = t->zs[index - 1];
    for (int i = index - 1; i >= 0; --i) {
      double dz = zbase - t->zs[i];
      if (dz >= minSafety) break;
      safety = cone_safe_in(&t->sec[i], pcon_local(t, i, p));
      if (safety < minSafety) minSafety = safety;
    }
  }
  return minSafety;
}

/* SafetyToOut (PolyconeImplementation.h:452-517); the neighbouring sections are probed
 * with the cone's SafetyToIn, as the reference does */
static double polycone_safe_out(const or_polycone *t, v3 p)
{
  int cin = 0, cout = 0;
  polycone_ci(t, p, 1, &cin, &cout);
  if (cout) return -1;
  int index = polycone_section_index(t, p.z);
  if (index < 0) return -1;
  double safety    = cone_safe_out(&t->sec[index], pcon_local(t, index, p));
  double minSafety = safety;
  if (minSafety == kInfLength) return 0.;
  if (minSafety < kTolerance) return 0.;
  double zbase = t->zs[index + 1];
  for (int i = index + 1; i < t->nsec; ++i) {
    double dz = t->zs[i] - zbase;
    if (dz >= minSafety) break;
    safety = cone_safe_in(&t->sec[i], pcon_local(t, i, p));
    if (safety < minSafety) minSafety = safety;
  }
  if (index > 0) {
    zbase = t->zs[index - 1];
    for (int i = index - 1; i >= 0; --i) {
      double dz = zbase - t->zs[i];
      if (dz >= minSafety) break;
      safety = cone_safe_in(&t->sec[i], pcon_local(t, i, p));
      if (safety < minSafety) minSafety = safety;
    }
  }
  return minSafety;
}

/* UnplacedPolycone::Extent (source/UnplacedPolycone.cpp:865-902): z from the end planes,
 * x/y from Cone(minR, maxR, minR, maxR, 1, fStartPhi, fDeltaPhi) over the sections'
 * constructor radii */
static void polycone_extent(const or_polycone *t, v3 *mn, v3 *mx)
{
  double maxR = 0, minR = kInfLength;
  for (int i = 0; i < t->nsec; i++) {
    const or_cone *c = &t->sec[i];
    maxR             = or_max(maxR, or_max(c->o_rmax1, c->o_rmax2));
    minR             = or_min(minR, or_min(c->o_rmin1, c->o_rmin2));
  }
  double minz, maxz;
  if (t->zs[0] > t->zs[t->nsec]) {
    maxz = t->zs[0];
    minz = t->zs[t->nsec];
  } else {
    minz = t->zs[0];
    maxz = t->zs[t->nsec];
  }
  or_cone tmp;
  double cpar[7] = {minR, maxR, minR, maxR, 1, t->startPhi, t->deltaPhi};
  cone_init(&tmp, cpar, NULL, 0);
  cone_extent(&tmp, mn, mx);
  mn->z = minz;
  mx->z = maxz;
}

/* ================================================================== */
/* dispatch                                                           */
/* ================================================================== */
/* Orb (OrbImplementation.h:60-225, OrbStruct.h:19-25, source/UnplacedOrb.cpp:58-63)    */

/* GenericKernelForContainsAndInside (OrbImplementation.h:88-100) */
static int orb_contains(const or_orb *o, v3 p)
{
  double rad2 = v3_mag2(p);
  double tolR = o->r + kTolerance;
  return !(rad2 >= tolR * tolR);
}

static int orb_inside(const or_orb *o, v3 p) /* OrbImplementation.h:72-85 */
{
  double rad2 = v3_mag2(p);
  double tolR = o->r - kTolerance;
  int cin     = rad2 <= tolR * tolR;
  int cout;
  tolR = o->r + kTolerance;
  cout = rad2 >= tolR * tolR;
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

/* DetectIntersectionAndCalculateDistance (OrbImplementation.h:197-220) */
static int orb_intersect(const or_orb *o, v3 p, v3 d, int toIn, double *dist)
{
  double rad2    = v3_mag2(p);
  double pDotV3D = v3_dot(p, d);
  double c       = rad2 - o->r * o->r;
  double d2      = pDotV3D * pDotV3D - c;
  if (toIn) {
    if (d2 >= 0. && pDotV3D <= 0.) {
      *dist = -pDotV3D - sqrt(fabs(d2));
      return 1;
    }
    return 0;
  }
  if (d2 >= 0.) {
    *dist = -pDotV3D + sqrt(fabs(d2));
    return 1;
  }
  return 0;
}

static double orb_dist_in(const or_orb *o, v3 p, v3 d) /* OrbImplementation.h:102-124 */
{
  double rad = sqrt(v3_mag2(p)), pDotV3D, dist = kInfLength;
  if (rad < o->r - kTolerance) return -1.;
  pDotV3D = v3_dot(p, d);
  if (rad >= o->r - kTolerance && rad <= o->r + kTolerance && pDotV3D < 0.) return 0.;
  return orb_intersect(o, p, d, 1, &dist) ? dist : kInfLength;
}

static double orb_dist_out(const or_orb *o, v3 p, v3 d) /* OrbImplementation.h:126-150 */
{
  double rad = sqrt(v3_mag2(p)), pDotV3D, dist = kInfLength;
  if (rad > o->r + kTolerance) return -1.;
  pDotV3D = v3_dot(p, d);
  if (rad >= o->r - kTolerance && rad <= o->r + kTolerance && pDotV3D > 0.) return 0.;
  return orb_intersect(o, p, d, 0, &dist) ? dist : kInfLength;
}

static double orb_safe_in(const or_orb *o, v3 p) /* OrbImplementation.h:152-165 */
{
  double rad    = sqrt(v3_mag2(p));
  double safety = rad - o->r;
  if (rad < o->r - kTolerance) return -1.;
  if (rad > o->r - kTolerance && rad < o->r + kTolerance) safety = 0.;
  return safety;
}

static double orb_safe_out(const or_orb *o, v3 p) /* OrbImplementation.h:167-181 */
{
  double rad    = sqrt(v3_mag2(p));
  double safety = o->r - rad;
  if (rad > o->r + kTolerance) return -1.;
  if (rad > o->r - kTolerance && rad < o->r + kTolerance) safety = 0.;
  return safety;
}

/* ================================================================== */
/* CutTube (CutTubeImplementation.h:101-290, CutTubeStruct.h:21-46, CutPlanes.h:95-170,
 * Plane.h:44-191, source/UnplacedCutTube.cpp:128-172)                                  */

/* Plane::Set(normal, origin) (Plane.h:44-51) with Vector3D::FixZeroes (Vector3D.h:298-305) */
static void plane_set(or_plane *pl, v3 normal, v3 origin)
{
  v3 f = normal;
  double inv;
  if (fabs(f.x) < kTolerance) f.x = 0.0;
  if (fabs(f.y) < kTolerance) f.y = 0.0;
  if (fabs(f.z) < kTolerance) f.z = 0.0;
  inv      = 1. / sqrt(v3_mag2(f));
  pl->n[0] = inv * f.x;
  pl->n[1] = inv * f.y;
  pl->n[2] = inv * f.z;
  pl->d    = inv * -v3_dot(f, origin);
}

static inline double plane_dist(const or_plane *pl, v3 p) /* DistPlane (Plane.h:102-107) */
{
  return p.x * pl->n[0] + p.y * pl->n[1] + p.z * pl->n[2] + pl->d;
}

static inline double plane_ndd(const or_plane *pl, v3 d) { return NonZero(d.x * pl->n[0] + d.y * pl->n[1] + d.z * pl->n[2]); }

static double plane_dist_in(const or_plane *pl, v3 p, v3 d) /* Plane.h:131-147 */
{
  double ndd = plane_ndd(pl, d), saf = plane_dist(pl, p);
  if (ndd < 0. && saf > -kTolerance) return -saf / ndd;
  return -kInfLength;
}

static double plane_dist_out(const or_plane *pl, v3 p, v3 d) /* Plane.h:152-171 */
{
  double ndd = plane_ndd(pl, d), saf = plane_dist(pl, p), distance = kInfLength;
  int valid = ndd > 0. && saf < kTolerance;
  if (saf > kTolerance) distance = -kInfLength;
  if (valid) distance = -saf / ndd;
  return distance;
}

static int cutplanes_contains(const or_cuttube *c, v3 p) /* CutPlanes.h:101-105 */
{
  return plane_dist(&c->cut[0], p) < 0. && plane_dist(&c->cut[1], p) < 0.;
}

static int cutplanes_inside(const or_cuttube *c, v3 p) /* CutPlanes.h:107-119 */
{
  double d0 = plane_dist(&c->cut[0], p), d1 = plane_dist(&c->cut[1], p);
  int inside = (d0 < 0.0 && d1 < 0.0) ? kInsideE : kOutsideE;
  if (fabs(d0) < kTolerance || fabs(d1) < kTolerance) inside = kSurfaceE;
  return inside;
}

static double cutplanes_dist_in(const or_cuttube *c, v3 p, v3 d) /* CutPlanes.h:121-136 */
{
  double d0 = plane_dist_in(&c->cut[0], p, d), d1;
  if (d.x * c->cut[0].n[0] + d.y * c->cut[0].n[1] + d.z * c->cut[0].n[2] > 0.) d0 = -kInfLength;
  d1 = plane_dist_in(&c->cut[1], p, d);
  if (d.x * c->cut[1].n[0] + d.y * c->cut[1].n[1] + d.z * c->cut[1].n[2] > 0.) d1 = -kInfLength;
  return or_max(d0, d1);
}

static double cutplanes_dist_out(const or_cuttube *c, v3 p, v3 d) /* CutPlanes.h:138-146 */
{
  return or_min(plane_dist_out(&c->cut[0], p, d), plane_dist_out(&c->cut[1], p, d));
}

static double cutplanes_safe_in(const or_cuttube *c, v3 p) /* CutPlanes.h:148-156 */
{
  return or_max(plane_dist(&c->cut[0], p), plane_dist(&c->cut[1], p));
}

static double cutplanes_safe_out(const or_cuttube *c, v3 p) /* CutPlanes.h:158-166 */
{
  return or_min(-plane_dist(&c->cut[0], p), -plane_dist(&c->cut[1], p));
}

/* Vector3D::Unit (Vector3D.h:284-290) */
static v3 v3_unit(v3 a)
{
  double m = sqrt(v3_mag2(a) + 2.2250738585072014e-308); /* + kMinimum */
  return v3_make(a.x / m, a.y / m, a.z / m);
}

/* UnplacedCutTube(rmin, rmax, z, sphi, dphi, bx, by, bz, tx, ty, tz) -> CutTubeStruct
 * (UnplacedCutTube.h:54-70, CutTubeStruct.h:34-46) */
static int cuttube_init(or_cuttube *c, const double *a, char *err, int errlen)
{
  double tp[5];
  v3 bn = v3_make(a[5], a[6], a[7]), tn = v3_make(a[8], a[9], a[10]);
  if (bn.z >= 0 || tn.z <= 0) {
    set_err(err, errlen, "cut tube: illegal normal direction for cut planes");
    return -1;
  }
  tp[0] = a[0];
  tp[1] = a[1];
  tp[2] = kInfLength; /* the tube of a cut tube has an infinite half-length */
  tp[3] = a[3];
  tp[4] = a[4];
  if (tube_init(&c->tube, tp, err, errlen)) return -1;
  c->dz = a[2];
  plane_set(&c->cut[0], v3_unit(bn), v3_make(0., 0., -a[2]));
  plane_set(&c->cut[1], v3_unit(tn), v3_make(0., 0., a[2]));
  c->cosphi1 = cos(a[3]);
  c->sinphi1 = sin(a[3]);
  c->cosphi2 = cos(a[3] + a[4]);
  c->sinphi2 = sin(a[3] + a[4]);
  c->maxval  = or_max(a[1], a[2]);
  return 0;
}

static int cuttube_contains(const or_cuttube *c, v3 p) /* CutTubeImplementation.h:101-113 */
{
  if (!cutplanes_contains(c, p)) return 0; /* EarlyReturnAllowed */
  return tube_contains(&c->tube, p);
}

static int cuttube_inside(const or_cuttube *c, v3 p) /* CutTubeImplementation.h:115-130 */
{
  int incp = cutplanes_inside(c, p), inside;
  if (incp == kOutsideE) return kOutsideE; /* MaskFull(inside_cutplanes == kOutside) */
  inside = tube_inside(&c->tube, p);
  if (incp == kOutsideE || (incp == kSurfaceE && inside != kOutsideE)) inside = incp;
  return inside;
}

/* DistanceToInKernel (CutTubeImplementation.h:158-245) */
static double cuttube_dist_in_kernel(const or_cuttube *c, v3 p, v3 d, double stepmax)
{
  double distance = kInfLength, dplanes, safplanes, dexit, dtube;
  int incp, instart, hitplanes, done, inside;
  v3 prop;
  incp    = cutplanes_inside(c, p);
  instart = tube_inside(&c->tube, p);
  if (incp == kOutsideE || (incp == kSurfaceE && instart != kOutsideE)) instart = incp;
  if (instart == kInsideE) distance = -1.;
  dplanes   = cutplanes_dist_in(c, p, d);
  safplanes = cutplanes_safe_in(c, p);
  hitplanes = fabs(dplanes) < stepmax && safplanes > -kTolerance;
  if (incp != kInsideE && !hitplanes) return distance;
  prop = p;
  if (!hitplanes) dplanes = 0.;
  if (hitplanes) {
    prop = v3_add(prop, v3_scale(dplanes, d));
    incp = cutplanes_inside(c, prop);
  }
  done = incp == kOutsideE;
  done |= instart == kInsideE;
  if (done) return distance;
  instart = tube_inside(&c->tube, prop);
  inside  = hitplanes && instart != kOutsideE;
  if (inside && !done) distance = dplanes;
  done |= inside;
  if (done) {
    if (fabs(distance) < kTolerance) distance = 0.;
    return distance;
  }
  dexit = cutplanes_dist_out(c, prop, d);
  dtube = tube_dist_in_kernel(&c->tube, prop, d);
  if (dtube < 0.) dtube = 0.;
  if (dexit < dtube) dtube = kInfLength;
  if (!done && (dtube + dplanes) < stepmax) distance = dtube + dplanes;
  return distance;
}

/* DistanceToIn with the far-point pre-move (CutTubeImplementation.h:132-156) */
static double cuttube_dist_in(const or_cuttube *c, v3 pt, v3 d, double stepmax)
{
  v3 p          = pt;
  double ptDist = sqrt(v3_mag2(p)), distToMove = 0., distance;
  const double order = 100.;
  if (ptDist > order * c->maxval) {
    distToMove = ptDist - order * c->maxval;
    p          = v3_add(p, v3_scale(distToMove, d));
  }
  distance = cuttube_dist_in_kernel(c, p, d, stepmax);
  distance += distToMove;
  return distance;
}

static double cuttube_dist_out(const or_cuttube *c, v3 p, v3 d) /* CutTubeImplementation.h:247-259 */
{
  double distance = cutplanes_dist_out(c, p, d);
  double dtube    = tube_dist_out(&c->tube, p, d);
  if (dtube < distance) distance = dtube;
  return distance;
}

static double cuttube_safe_in(const or_cuttube *c, v3 p) /* CutTubeImplementation.h:261-269 */
{
  double safety = cutplanes_safe_in(c, p), saftube = tube_safe_in(&c->tube, p);
  if (saftube > safety) safety = saftube;
  return safety;
}

static double cuttube_safe_out(const or_cuttube *c, v3 p) /* CutTubeImplementation.h:271-279 */
{
  double safety = cutplanes_safe_out(c, p), saftube = tube_safe_out(&c->tube, p);
  if (saftube < safety) safety = saftube;
  return safety;
}

/* ZlimitTop / ZlimitBottom (UnplacedCutTube.h:135-147) */
static double cuttube_zlimit(const or_cuttube *c, int top, double rval, double phival)
{
  const double *n = c->cut[top].n;
  return (top ? c->dz : -c->dz) - (rval / n[2]) * (n[0] * cos(phival) + n[1] * sin(phival));
}

static void cuttube_extent(const or_cuttube *c, v3 *mn, v3 *mx) /* source/UnplacedCutTube.cpp:128-172 */
{
  const or_tube *t = &c->tube;
  const double *bn = c->cut[0].n, *tn = c->cut[1].n;
  double dztop    = t->rmax * sqrt(1. - tn[2] * tn[2]) / tn[2];
  double dzbottom = -t->rmax * sqrt(1. - bn[2] * bn[2]) / bn[2];
  *mn = v3_make(-t->rmax, -t->rmax, -c->dz - dzbottom);
  *mx = v3_make(t->rmax, t->rmax, c->dz + dztop);
  if (t->dphi == kTwoPi) return;
  if (!wedge_contains(&t->w, v3_make(-tn[0], -tn[1], 0.))) {
    mx->z = or_max(cuttube_zlimit(c, 1, t->rmax, t->sphi), cuttube_zlimit(c, 1, t->rmax, t->sphi + t->dphi));
    mx->z = or_max(mx->z, or_max(cuttube_zlimit(c, 1, t->rmin, t->sphi), cuttube_zlimit(c, 1, t->rmin, t->sphi + t->dphi)));
  }
  if (!wedge_contains(&t->w, v3_make(-bn[0], -bn[1], 0.))) {
    mn->z = or_min(cuttube_zlimit(c, 0, t->rmax, t->sphi), cuttube_zlimit(c, 0, t->rmax, t->sphi + t->dphi));
    mn->z = or_min(mn->z, or_min(cuttube_zlimit(c, 0, t->rmin, t->sphi), cuttube_zlimit(c, 0, t->rmin, t->sphi + t->dphi)));
  }
  if (!wedge_contains(&t->w, v3_make(1., 0., 0.))) {
    mx->x = or_max(t->rmax * c->cosphi1, t->rmax * c->cosphi2);
    mx->x = or_max(mx->x, or_max(t->rmin * c->cosphi1, t->rmin * c->cosphi2));
  }
  if (!wedge_contains(&t->w, v3_make(-1., 0., 0.))) {
    mn->x = or_min(t->rmax * c->cosphi1, t->rmax * c->cosphi2);
    mn->x = or_min(mn->x, or_min(t->rmin * c->cosphi1, t->rmin * c->cosphi2));
  }
  if (!wedge_contains(&t->w, v3_make(0., 1., 0.))) {
    mx->y = or_max(t->rmax * c->sinphi1, t->rmax * c->sinphi2);
    mx->y = or_max(mx->y, or_max(t->rmin * c->sinphi1, t->rmin * c->sinphi2));
  }
  if (!wedge_contains(&t->w, v3_make(0., -1., 0.))) {
    mn->y = or_min(t->rmax * c->sinphi1, t->rmax * c->sinphi2);
    mn->y = or_min(mn->y, or_min(t->rmin * c->sinphi1, t->rmin * c->sinphi2));
  }
}

/* ================================================================== */

/* ================================================================== */
/* Polyhedron: PolyhedronStruct.h, Quadrilaterals.h/.cpp, Planes.h/.cpp,
 * kernel/PolyhedronImplementation.h.  The specialisation the reference builds for a
 * placement (UnplacedPolyhedron.cpp:75-103: inner radii and phi cut-out kinds chosen from
 * the shape) behaves as the generic one with the shape's own flags, which is what is
 * restated here.                                                     */
/* ================================================================== */

/* NormalizeAngle<kScalar> (GenericKernels.h:140-146) */
static double phd_normalize_angle(double a) { return a + kTwoPi * (double)((a < 0) - (int)(a / kTwoPi)); }

/* Vector3D::FixZeroes (Vector3D.h:298-305) */
static v3 v3_fix_zeroes(v3 a)
{
  if (fabs(a.x) < kTolerance) a.x = 0.0;
  if (fabs(a.y) < kTolerance) a.y = 0.0;
  if (fabs(a.z) < kTolerance) a.z = 0.0;
  return a;
}

/* Vector3D::Normalized (Vector3D.h:202): v * (1 / Length()) */
static v3 v3_normalized(v3 a)
{
  const double inv = 1. / sqrt(v3_mag2(a));
  return v3_make(a.x * inv, a.y * inv, a.z * inv);
}

/* operator== of Vector3D<Precision> (Vector3D.h:387-390): componentwise within kTolerance */
static int v3_tol_eq(v3 a, v3 b)
{
  return fabs(a.x - b.x) < kTolerance && fabs(a.y - b.y) < kTolerance && fabs(a.z - b.z) < kTolerance;
}

static inline v3 quad_corner(const or_quad *q, int j) { return v3_make(q->c[j][0], q->c[j][1], q->c[j][2]); }
static inline v3 quad_normal(const or_quad *q) { return v3_make(q->n[0], q->n[1], q->n[2]); }
static inline v3 quad_side(const or_quad *q, int j) { return v3_make(q->sn[j][0], q->sn[j][1], q->sn[j][2]); }

/* Planes::Set(index, normal, origin) (source/Planes.cpp:30-37) of one side plane */
static void quad_set_side(or_quad *q, int j, v3 normal, v3 origin)
{
  const v3 fixed   = v3_fix_zeroes(normal);
  const double inv = 1. / sqrt(v3_mag2(fixed));
  q->sn[j][0] = inv * fixed.x;
  q->sn[j][1] = inv * fixed.y;
  q->sn[j][2] = inv * fixed.z;
  q->sd[j]    = inv * -v3_dot(fixed, origin);
}

/* Quadrilaterals::Set (source/Quadrilaterals.cpp:33-104); -1 when fewer than three corners are
 * distinct (the reference then reads an unset corner) */
static int quad_set(or_quad *q, v3 c0, v3 c1, v3 c2, v3 c3)
{
  const v3 in[4] = {c0, c1, c2, c3};
  v3 ch[4];
  int assigned = 1, tested = 1, j;
  double a, b, c, d, inv;
  v3 normal;
  for (j = 0; j < 4; ++j) {
    q->c[j][0] = in[j].x;
    q->c[j][1] = in[j].y;
    q->c[j][2] = in[j].z;
  }
  ch[0] = in[0];
  while (tested < 4) {
    int chosen = 1;
    for (j = 0; j < assigned; ++j)
      if (v3_tol_eq(ch[j], in[tested])) {
        chosen = 0;
        break;
      }
    if (chosen) ch[assigned++] = in[tested];
    ++tested;
  }
  if (assigned < 3) return -1;
  a = ch[0].y * (ch[1].z - ch[2].z) + ch[1].y * (ch[2].z - ch[0].z) + ch[2].y * (ch[0].z - ch[1].z);
  b = ch[0].z * (ch[1].x - ch[2].x) + ch[1].z * (ch[2].x - ch[0].x) + ch[2].z * (ch[0].x - ch[1].x);
  c = ch[0].x * (ch[1].y - ch[2].y) + ch[1].x * (ch[2].y - ch[0].y) + ch[2].x * (ch[0].y - ch[1].y);
  d = -ch[0].x * (ch[1].y * ch[2].z - ch[2].y * ch[1].z) - ch[1].x * (ch[2].y * ch[0].z - ch[0].y * ch[2].z) -
      ch[2].x * (ch[0].y * ch[1].z - ch[1].y * ch[0].z);
  normal = v3_make(a, b, c);
  inv    = 1. / sqrt(v3_mag2(normal));
  normal = v3_make(normal.x * inv, normal.y * inv, normal.z * inv);
  d *= inv;
  normal  = v3_fix_zeroes(normal);
  q->n[0] = normal.x;
  q->n[1] = normal.y;
  q->n[2] = normal.z;
  q->d    = d;
  for (j = 0; j < 4; ++j) {
    const v3 s0 = in[j], s1 = in[(j + 1) % 4];
    if (!v3_tol_eq(s1, s0)) {
      quad_set_side(q, j, v3_normalized(v3_cross(normal, v3_sub(s1, s0))), s0);
    } else {
      q->sn[j][0] = q->sn[j][1] = q->sn[j][2] = 0.;
      q->sd[j]                                = 0.;
    }
  }
  return 0;
}

/* Quadrilaterals::FlipSign -> Planes::FlipSign (source/Planes.cpp:45-49) */
static void quad_flip(or_quad *q)
{
  q->n[0] = -q->n[0];
  q->n[1] = -q->n[1];
  q->n[2] = -q->n[2];
  q->d    = -q->d;
}

/* Quadrilaterals::RayHitsQuadrilateral (Quadrilaterals.h:139-150) */
static int quad_ray_hits(const or_quad *q, v3 x)
{
  int j;
  for (j = 0; j < 4; ++j)
    if (!(v3_dot(x, quad_side(q, j)) + q->sd[j] >= -kTolerance)) return 0;
  return 1;
}

/* Quadrilaterals::DistanceToIn<double, behindPlanesT> (Quadrilaterals.h:361-396) */
static double quads_dist_in(const or_quads *qs, int behind, v3 p, v3 d)
{
  double best = kInfLength;
  int i;
  for (i = 0; i < qs->n; ++i) {
    const or_quad *q = &qs->q[i];
    const v3 n       = quad_normal(q);
    double dist      = v3_dot(p, n) + q->d;
    double proj;
    v3 x;
    if (!((behind ? -dist : dist) > -kTolerance)) continue;
    proj = v3_dot(d, n);
    if (!((behind ? proj : -proj) > 0)) continue;
    dist /= -(proj + copysign(1E-20, proj));
    x = v3_add(p, v3_scale(dist, d));
    if (quad_ray_hits(q, x)) best = dist;
    if (best < kInfLength) break;
  }
  return 0. > best ? 0. : best;
}

/* Quadrilaterals::DistanceToOut(point, direction, zMin, zMax) (Quadrilaterals.h:466-516) */
static double quads_dist_out(const or_quads *qs, v3 p, v3 d, double zMin, double zMax)
{
  double best = kInfLength;
  int i;
  for (i = 0; i < qs->n; ++i) {
    const or_quad *q = &qs->q[i];
    const v3 n       = quad_normal(q);
    double dt        = v3_dot(p, n) + q->d, proj;
    int valid;
    if (!(dt < kTolerance)) continue;
    proj = v3_dot(d, n);
    if (!(proj > 0)) continue;
    dt /= -proj;
    if (!(dt < best)) continue;
    if (zMin == zMax) {
      valid = quad_ray_hits(q, v3_add(p, v3_scale(dt, d)));
    } else {
      const double zp = p.z + dt * d.z;
      valid           = (zp >= zMin - kTolerance) && (zp < zMax + kTolerance);
    }
    if (!valid) continue;
    best = dt;
  }
  if (best > -kTolerance) best = best > 0. ? best : 0.;
  return best;
}

/* DistanceToLineSegmentSquared1 (GenericKernels.h:188-215) */
static double phd_segment_dist2(v3 c0, v3 c1, v3 p)
{
  double result = kInfLength, dot0, dot1;
  const v3 line = v3_sub(c1, c0);
  dot0          = v3_dot(v3_sub(p, c0), line);
  if (dot0 <= 0) return v3_mag2(v3_sub(p, c0));
  dot1 = v3_mag2(line);
  if (dot1 <= dot0) result = v3_mag2(v3_sub(p, c1));
  if (result < kInfLength) return result;
  return v3_mag2(v3_sub(v3_add(c0, v3_scale(dot0 / dot1, line)), p));
}

/* Quadrilaterals::ScalarDistanceSquared (Quadrilaterals.h:535-572) */
static double quad_dist2(const or_quad *q, v3 p)
{
  const v3 n      = quad_normal(q);
  double distance = v3_dot(p, n) + q->d, dsq = kInfLength;
  const v3 x      = v3_sub(p, v3_scale(distance, n));
  int within[4], j;
  for (j = 0; j < 4; ++j)
    within[j] = x.x * q->sn[j][0] + x.y * q->sn[j][1] + x.z * q->sn[j][2] + q->sd[j] >= 0;
  if (within[0] && within[1] && within[2] && within[3]) return distance * distance;
  for (j = 0; j < 4; ++j) {
    if (!within[j]) {
      distance = phd_segment_dist2(quad_corner(q, j), quad_corner(q, (j + 1) % 4), p);
      if (distance < dsq) dsq = distance;
    }
  }
  return dsq;
}

/* Planes::Contains (Planes.h:192-205) */
static int quads_contains(const or_quads *qs, v3 p)
{
  int i, r = 1;
  for (i = 0; i < qs->n; ++i) r &= v3_dot(p, quad_normal(&qs->q[i])) + qs->q[i].d < 0;
  return r;
}

/* Planes::Inside of one plane (Planes.h:268-281) */
static int quad_inside(const or_quad *q, v3 p)
{
  const double dist = q->n[0] * p.x + q->n[1] * p.y + q->n[2] * p.z + q->d;
  if (dist > kHalfTolerance) return kOutsideE;
  if (dist > -kHalfTolerance) return kSurfaceE;
  return kInsideE;
}

/* Planes::Inside over all planes (Planes.h:246-266) */
static int quads_inside(const or_quads *qs, v3 p)
{
  int i, r = kInsideE;
  for (i = 0; i < qs->n; ++i) {
    const double dist = qs->q[i].n[0] * p.x + qs->q[i].n[1] * p.y + qs->q[i].n[2] * p.z + qs->q[i].d;
    if (dist > kHalfTolerance) r = kOutsideE;
    if (r == kInsideE && dist > -kHalfTolerance) r = kSurfaceE;
    if (r == kOutsideE) break;
  }
  return r;
}

static int phd_alloc_quads(or_quads *qs, int n)
{
  qs->n = n;
  qs->q = n > 0 ? (or_quad *)calloc((size_t)n, sizeof(or_quad)) : NULL;
  return n > 0 && !qs->q ? -1 : 0;
}

void polyhedron_free(or_polyhedron *t)
{
  int i;
  if (t->seg)
    for (i = 0; i < t->nz - 1; ++i) {
      free(t->seg[i].outer.q);
      free(t->seg[i].phi.q);
      free(t->seg[i].inner.q);
    }
  free(t->seg);
  free(t->z);
  free(t->rmin);
  free(t->rmax);
  free(t->samez);
  free(t->phisec);
  t->seg = NULL;
  t->z = t->rmin = t->rmax = NULL;
  t->samez  = NULL;
  t->phisec = NULL;
}

/* PolyhedronStruct(phiStart, phiDelta, sideCount, zPlaneCount, zPlanes, rMin, rMax) and
 * Initialize (PolyhedronStruct.h:96-110, 264-420); params: sphi, dphi, sides, nz, z[nz],
 * rmin[nz], rmax[nz].  Refused where the reference would read past its arrays: zero-length
 * first or last segment, three equal z planes in a row, a zero-length segment whose faces
 * are all empty, a face with fewer than three distinct corners. */
static int polyhedron_init(or_polyhedron *t, const double *a, char *err, int errlen)
{
  const double phiStart0 = a[0], phiDelta0 = a[1];
  const int S = (int)a[2], nz = (int)a[3];
  const double *zp = a + 4, *rmn = a + 4 + nz, *rmx = a + 4 + 2 * nz;
  double phiStart, phiDelta, sidePhi, cosHalf, inner = kInfLength, outer = -kInfLength, tp[5];
  int i, iPlane, iSide;
  memset(t, 0, sizeof(*t));
  if (!(phiDelta0 > 0) || S < 1 || nz < 2 || !((phiDelta0 > kTwoPi ? kTwoPi : phiDelta0) / S < kPi)) {
    set_err(err, errlen, "polyhedron: needs dphi > 0, nz >= 2 and sides with dphi / sides < pi");
    return -1;
  }
  for (i = 0; i < nz; ++i) {
    if (!(rmn[i] >= 0 && rmx[i] >= rmn[i]) || (i > 0 && !(zp[i] >= zp[i - 1]))) {
      set_err(err, errlen, "polyhedron: needs 0 <= rmin <= rmax and non-decreasing z planes");
      return -1;
    }
    if (i + 2 < nz && zp[i] == zp[i + 1] && zp[i + 1] == zp[i + 2]) {
      set_err(err, errlen, "polyhedron: three equal z planes in a row");
      return -1;
    }
  }
  if (zp[0] == zp[1] || zp[nz - 2] == zp[nz - 1]) {
    set_err(err, errlen, "polyhedron: zero-length first or last segment");
    return -1;
  }
  t->sides       = S;
  t->nz          = nz;
  t->hasPhi      = phiDelta0 < kTwoPi;
  t->hasLargePhi = phiDelta0 < kPi;
  t->phiStart    = phd_normalize_angle(phiStart0);
  t->phiDelta    = phiDelta0 > kTwoPi ? kTwoPi : phiDelta0;
  wedge_init(&t->w, t->phiDelta, t->phiStart);
  t->seg    = (or_zseg *)calloc((size_t)(nz - 1), sizeof(or_zseg));
  t->z      = (double *)malloc(sizeof(double) * (size_t)nz);
  t->rmin   = (double *)malloc(sizeof(double) * (size_t)nz);
  t->rmax   = (double *)malloc(sizeof(double) * (size_t)nz);
  t->samez  = (int *)calloc((size_t)nz, sizeof(int));
  t->phisec = (v3 *)malloc(sizeof(v3) * (size_t)(S + 1));
  if (!t->seg || !t->z || !t->rmin || !t->rmax || !t->samez || !t->phisec) goto nomem;
  for (i = 0; i < nz; ++i) {
    t->z[i]    = zp[i];
    t->rmin[i] = rmn[i];
    t->rmax[i] = rmx[i];
    if (i > 0 && i < nz - 1 && zp[i] == zp[i + 1]) t->samez[i] = 1;
  }
  for (i = 0; i < nz - 1; ++i) {
    const int hasInnerRadius = rmn[i] > 0 || rmn[i + 1] > 0;
    int mult                 = (zp[i] == zp[i + 1] && rmx[i] == rmx[i + 1]) ? 0 : 1;
    if (phd_alloc_quads(&t->seg[i].outer, S * mult)) goto nomem;
    if (t->hasPhi && phd_alloc_quads(&t->seg[i].phi, zp[i] == zp[i + 1] ? 0 : 2)) goto nomem;
    mult = (zp[i] == zp[i + 1] && rmn[i] == rmn[i + 1]) ? 0 : 1;
    if (hasInnerRadius && mult > 0) {
      if (phd_alloc_quads(&t->seg[i].inner, S)) goto nomem;
      t->hasInner = 1;
    }
    if (zp[i] == zp[i + 1] && t->seg[i].outer.n == 0 && t->seg[i].inner.n == 0) {
      set_err(err, errlen, "polyhedron: a zero-length segment needs different radii on its two planes");
      polyhedron_free(t);
      return -1;
    }
  }
  phiStart = phd_normalize_angle(phiStart0);
  phiDelta = phiDelta0 > kTwoPi ? kTwoPi : phiDelta0;
  sidePhi  = phiDelta / S;
#define PHD_PHI(side) phd_normalize_angle(phiStart + ((!t->hasPhi && (side) == S) ? 0 : (side)) * sidePhi)
  for (i = 0; i <= S; ++i) {
    const double phi = PHD_PHI(i);
    const v3 corner  = v3_fix_zeroes(v3_normalized(v3_make(1. * cos(phi), 1. * sin(phi), 0)));
    t->phisec[i]     = v3_cross(v3_normalized(corner), v3_make(0, 0, -1));
  }
  cosHalf = cos(0.5 * sidePhi);
  for (i = 0; i < nz; ++i) {
    if (rmn[i] < inner) inner = rmn[i];
    if (rmx[i] > outer) outer = rmx[i];
  }
  outer /= cosHalf;
  tp[0] = inner - kHalfTolerance;
  tp[1] = outer + kHalfTolerance;
  tp[2] = 0.5 * (zp[nz - 1] - zp[0]) + kTolerance;
  tp[3] = !t->hasPhi ? 0 : phiStart - 100 * kTolerance;
  tp[4] = !t->hasPhi ? kTwoPi : phiDelta + 2 * (100 * kTolerance);
  if (tube_init(&t->btube, tp, err, errlen)) {
    polyhedron_free(t);
    return -1;
  }
  t->btubeOffset = 0.5 * (zp[0] + zp[nz - 1]);
#define PHD_VTX(r, i, j) \
  v3_fix_zeroes(v3_make((r)[i] / cosHalf * cos(PHD_PHI(j)), (r)[i] / cosHalf * sin(PHD_PHI(j)), zp[i]))
  for (iPlane = 0; iPlane < nz - 1; ++iPlane) {
    or_zseg *sg = &t->seg[iPlane];
    for (iSide = 0; iSide < sg->outer.n; ++iSide) {
      const v3 c0 = PHD_VTX(rmx, iPlane, iSide);
      or_quad *q  = &sg->outer.q[iSide];
      if (quad_set(q, c0, PHD_VTX(rmx, iPlane, iSide + 1), PHD_VTX(rmx, iPlane + 1, iSide + 1),
                   PHD_VTX(rmx, iPlane + 1, iSide)))
        goto degenerate;
      if (q->n[0] * c0.x + q->n[1] * c0.y < 0) quad_flip(q);
    }
    for (iSide = 0; iSide < sg->inner.n; ++iSide) {
      const v3 c0 = PHD_VTX(rmn, iPlane, iSide);
      or_quad *q  = &sg->inner.q[iSide];
      if (quad_set(q, c0, PHD_VTX(rmn, iPlane, iSide + 1), PHD_VTX(rmn, iPlane + 1, iSide + 1),
                   PHD_VTX(rmn, iPlane + 1, iSide)))
        goto degenerate;
      if (q->n[0] * c0.x + q->n[1] * c0.y < 0) quad_flip(q);
    }
    if (t->hasPhi && sg->phi.n == 2) {
      if (quad_set(&sg->phi.q[0], PHD_VTX(rmn, iPlane, 0), PHD_VTX(rmn, iPlane + 1, 0), PHD_VTX(rmx, iPlane + 1, 0),
                   PHD_VTX(rmx, iPlane, 0)))
        goto degenerate;
      if (v3_dot(quad_normal(&sg->phi.q[0]), t->phisec[0]) > 0) quad_flip(&sg->phi.q[0]);
      if (quad_set(&sg->phi.q[1], PHD_VTX(rmx, iPlane, S), PHD_VTX(rmx, iPlane + 1, S), PHD_VTX(rmn, iPlane + 1, S),
                   PHD_VTX(rmn, iPlane, S)))
        goto degenerate;
      if (v3_dot(quad_normal(&sg->phi.q[1]), t->phisec[S]) < 0) quad_flip(&sg->phi.q[1]);
    }
  }
#undef PHD_VTX
#undef PHD_PHI
  return 0;
degenerate:
  set_err(err, errlen, "polyhedron: a face has fewer than three distinct corners");
  polyhedron_free(t);
  return -1;
nomem:
  set_err(err, errlen, "polyhedron: out of host memory");
  polyhedron_free(t);
  return -1;
}

/* FindZSegmentKernel<double> (PolyhedronImplementation.h:232-244) */
static int phd_find_z(const or_polyhedron *t, double pz)
{
  int index = -1, b = 0;
  while (b < t->nz - 1 && pz - kTolerance > t->z[b]) {
    ++index;
    ++b;
  }
  if (pz + kTolerance > t->z[b]) return index + 1;
  return index;
}

/* FindPhiSegment (PolyhedronImplementation.h:256-276) */
static int phd_find_phi(const or_polyhedron *t, v3 p)
{
  int index = -1, i;
  double first = p.x * t->phisec[0].x + p.y * t->phisec[0].y + p.z * t->phisec[0].z, second;
  for (i = 1; i < t->sides + 1; ++i) {
    second = p.x * t->phisec[i].x + p.y * t->phisec[i].y + p.z * t->phisec[i].z;
    if (first > -kTolerance && second < kTolerance) index = i - 1;
    if (index >= 0) break;
    first = second;
  }
  return index;
}

static inline int phd_clamp_z(const or_polyhedron *t, int z)
{
  const int zmax = t->nz - 1;
  return z < 0 ? 0 : (z >= zmax ? zmax - 1 : z);
}

/* DistanceToInZSegment (PolyhedronImplementation.h:278-318) */
static double phd_dist_in_seg(const or_polyhedron *t, int si, v3 p, v3 d)
{
  const or_zseg *sg = &t->seg[si];
  double distance   = quads_dist_in(&sg->outer, 0, p, d);
  if (distance < kInfLength) return distance;
  if (t->hasPhi) distance = quads_dist_in(&sg->phi, 0, p, d);
  if (distance < kInfLength) return distance;
  if (sg->inner.n > 0) distance = quads_dist_in(&sg->inner, 1, p, d);
  return distance;
}

/* DistanceToOutZSegment (PolyhedronImplementation.h:320-362) */
static double phd_dist_out_seg(const or_polyhedron *t, int si, double zMin, double zMax, v3 p, v3 d)
{
  const or_zseg *sg = &t->seg[si];
  int done          = 0;
  double distance   = kInfLength;
  if (sg->inner.n > 0) {
    distance = quads_dist_in(&sg->inner, 0, p, d);
    done     = distance < kInfLength;
    if (done) return distance;
  }
  if (t->hasPhi) {
    const double distphi = quads_dist_in(&sg->phi, 1, p, d);
    if (!done && distance > -kTolerance) distance = distphi;
    done = distance > -kTolerance && distance < kInfLength;
    if (done) return distance;
  }
  {
    const double distout = quads_dist_out(&sg->outer, p, d, zMin, zMax);
    if (!done) distance = distout;
  }
  return distance;
}

/* InPhiCutoutWedge (PolyhedronImplementation.h:541-555) */
static int phd_in_cutout(const or_zseg *sg, int large, v3 p)
{
  const int s0 = v3_dot(p, quad_normal(&sg->phi.q[0])) + sg->phi.q[0].d >= 0;
  const int s1 = v3_dot(p, quad_normal(&sg->phi.q[1])) + sg->phi.q[1].d >= 0;
  return large ? (s0 || s1) : (s0 && s1);
}

/* ScalarSafetyToZSegmentSquared (PolyhedronImplementation.h:364-466); `phiIndex` may be moved
 * to the first or last side, as in the reference */
static double phd_safety_seg2(const or_polyhedron *t, int si, int *phiIndex, v3 p, int pt_inside)
{
  const or_zseg *sg = &t->seg[si];
  const int in_cutout = *phiIndex < 0;
  double s2           = kInfLength, so, sin_;
  if (t->hasPhi && sg->phi.n == 2) {
    if (pt_inside || in_cutout) {
      double saf;
      s2  = quad_dist2(&sg->phi.q[0], p);
      saf = quad_dist2(&sg->phi.q[1], p);
      if (saf < s2) s2 = saf;
      if (in_cutout) {
        if (t->hasLargePhi && sg->inner.n > 0) {
          sin_ = quad_dist2(&sg->inner.q[0], p);
          if (sin_ < s2) {
            *phiIndex = 0;
            s2        = sin_;
          }
          if (sg->inner.n > 1) {
            sin_ = quad_dist2(&sg->inner.q[sg->inner.n - 1], p);
            if (sin_ < s2) {
              *phiIndex = sg->inner.n - 1;
              s2        = sin_;
            }
          }
        }
        return s2;
      }
    }
  }
  if (in_cutout && si > 0 && si < t->nz - 2 && t->z[si] == t->z[si + 1]) {
    if (sg->outer.n > 0) {
      so = quad_dist2(&sg->outer.q[0], p);
      if (so < s2) {
        *phiIndex = 0;
        s2        = so;
      }
      if (sg->outer.n > 1) {
        so = quad_dist2(&sg->outer.q[sg->outer.n - 1], p);
        if (so < s2) {
          *phiIndex = sg->outer.n - 1;
          s2        = so;
        }
      }
    }
    if (sg->inner.n > 0) {
      sin_ = quad_dist2(&sg->inner.q[0], p);
      if (sin_ < s2) {
        *phiIndex = 0;
        s2        = sin_;
      }
      if (sg->inner.n > 1) {
        sin_ = quad_dist2(&sg->inner.q[sg->inner.n - 1], p);
        if (sin_ < s2) {
          *phiIndex = sg->inner.n - 1;
          s2        = sin_;
        }
      }
    }
    return s2;
  }
  so   = sg->outer.n > 0 ? quad_dist2(&sg->outer.q[*phiIndex], p) : kInfLength;
  sin_ = sg->inner.n > 0 ? quad_dist2(&sg->inner.q[*phiIndex], p) : kInfLength;
  if (sin_ < s2) s2 = sin_;
  if (so < s2) s2 = so;
  return s2;
}

/* ScalarDistanceToEndcaps<pointInsideT> (PolyhedronImplementation.h:468-511) */
static void phd_dist_endcaps(const or_polyhedron *t, int inside, v3 p, v3 d, double *distance)
{
  const int nseg = t->nz - 1;
  const int last = inside ? !(d.z < 0) : (d.z < 0);
  const or_zseg *sg = &t->seg[last ? nseg - 1 : 0];
  const double zPlane = t->z[last ? nseg : 0];
  const double dt     = (zPlane - p.z) / NonZero(d.z);
  v3 x;
  if (dt < -kTolerance || dt >= *distance) return;
  x = v3_add(p, v3_scale(dt, d));
  if (!quads_contains(&sg->outer, x)) return;
  if (sg->inner.n > 0 && quads_contains(&sg->inner, x)) return;
  if (t->hasPhi && phd_in_cutout(sg, t->hasLargePhi, x)) return;
  *distance = dt;
}

/* ScalarSafetyToEndcapsSquared (PolyhedronImplementation.h:513-539) */
static void phd_safety_endcaps2(const or_polyhedron *t, v3 p, double *dist2)
{
  const int nseg      = t->nz - 1;
  const double first  = t->z[0] - p.z;
  const double lastd  = t->z[nseg] - p.z;
  const int isFirst   = fabs(first) < fabs(lastd);
  const or_zseg *sg   = &t->seg[isFirst ? 0 : nseg - 1];
  const double dt     = isFirst ? first : lastd;
  const double dt2    = dt * dt;
  v3 x;
  if (dt2 >= *dist2) return;
  x = v3_make(p.x, p.y, p.z + dt);
  if (!quads_contains(&sg->outer, x)) return;
  if (sg->inner.n > 0 && quads_contains(&sg->inner, x)) return;
  if (t->hasPhi && phd_in_cutout(sg, t->hasLargePhi, x)) return;
  *dist2 = dt2;
}

/* ScalarInsideSegBorder (PolyhedronImplementation.h:628-664) */
static int phd_inside_border(const or_polyhedron *t, v3 p, int zi)
{
  const or_zseg *sg = &t->seg[zi];
  const int phiIndex = phd_find_phi(t, p);
  const or_quad *q;
  double r;
  int in1, in2;
  if (phiIndex < 0) return kOutsideE;
  q   = sg->outer.n ? &sg->outer.q[phiIndex] : &sg->inner.q[phiIndex];
  r   = fabs(v3_dot(p, quad_side(q, 0)));
  in1 = (r > t->rmin[zi] - kTolerance) && (r < t->rmax[zi] + kTolerance);
  in2 = (r > t->rmin[zi + 1] - kTolerance) && (r < t->rmax[zi + 1] + kTolerance);
  if (in1 && in2) {
    if ((r < t->rmin[zi] + kTolerance) || (r > t->rmax[zi] - kTolerance) || (r < t->rmin[zi + 1] + kTolerance) ||
        (r > t->rmax[zi + 1] - kTolerance))
      return kSurfaceE;
    if (t->hasPhi) {
      int cin = 0, cout = 0;
      wedge_ci(&t->w, p, 1, &cin, &cout);
      return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
    }
    return kInsideE;
  }
  if (!in1 && !in2) return kOutsideE;
  return kSurfaceE;
}

static inline int phd_wedge_inside(const or_wedge *w, v3 p) /* Wedge::Inside (Wedge_Evolution.h:262-272) */
{
  int cin = 0, cout = 0;
  wedge_ci(w, p, 1, &cin, &cout);
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

/* ScalarInsideSegPhi (PolyhedronImplementation.h:666-701) */
static int phd_inside_seg_phi(const or_polyhedron *t, v3 p, int zi, int phiIndex)
{
  const or_zseg *sg = &t->seg[zi];
  double dz;
  int r;
  if (phiIndex < 0) return kOutsideE;
  dz = fabs(p.z - t->btubeOffset) - 0.5 * (t->z[t->nz - 1] - t->z[0]);
  if (dz > kHalfTolerance) return kOutsideE;
  if (t->samez[zi]) return phd_inside_border(t, p, zi);
  r = quad_inside(&sg->outer.q[phiIndex], p);
  if (r != kInsideE) return r;
  if (sg->inner.n > 0) {
    r = quad_inside(&sg->inner.q[phiIndex], p);
    if (r == kInsideE) return kOutsideE;
    if (r == kSurfaceE) return kSurfaceE;
  }
  if (t->hasPhi) {
    r = phd_wedge_inside(&t->w, p);
    if (r != kInsideE) return r;
  }
  if (fabs(dz) < kHalfTolerance) return kSurfaceE;
  return kInsideE;
}

/* ScalarContainsKernel (PolyhedronImplementation.h:557-592) */
static int polyhedron_contains(const or_polyhedron *t, v3 p)
{
  int zi;
  const or_zseg *sg;
  if (!tube_contains(&t->btube, v3_make(p.x, p.y, p.z - t->btubeOffset))) return 0;
  zi = phd_find_z(t, p.z);
  if (!(zi >= 0 && zi < t->nz - 1)) return 0;
  sg = &t->seg[zi];
  if (t->samez[zi]) {
    const int phiIndex = phd_find_phi(t, p);
    const or_quad *q;
    double r;
    if (phiIndex < 0) return 0;
    q = sg->outer.n ? &sg->outer.q[phiIndex] : &sg->inner.q[phiIndex];
    r = fabs(v3_dot(p, quad_side(q, 0)));
    return ((r >= t->rmin[zi]) && (r <= t->rmax[zi])) | ((r >= t->rmin[zi + 1]) && (r <= t->rmax[zi + 1]));
  }
  if (!quads_contains(&sg->outer, p)) return 0;
  if (sg->inner.n > 0 && quads_contains(&sg->inner, p)) return 0;
  if (t->hasPhi && !quads_contains(&sg->phi, p)) return 0;
  return 1;
}

/* ScalarInsideKernel (PolyhedronImplementation.h:594-626) */
static int polyhedron_inside(const or_polyhedron *t, v3 p)
{
  int zi, r;
  const or_zseg *sg;
  double dz;
  if (!tube_contains(&t->btube, v3_make(p.x, p.y, p.z - t->btubeOffset))) return kOutsideE;
  zi = phd_find_z(t, p.z);
  if (zi > t->nz - 2) zi = t->nz - 2;
  if (zi < 0) zi = 0;
  sg = &t->seg[zi];
  if (t->samez[zi]) return phd_inside_border(t, p, zi);
  r = quads_inside(&sg->outer, p);
  if (r != kInsideE) return r;
  if (sg->inner.n > 0) {
    r = quads_inside(&sg->inner, p);
    if (r == kInsideE) return kOutsideE;
    if (r == kSurfaceE) return kSurfaceE;
  }
  if (t->hasPhi) {
    r = quads_inside(&sg->phi, p);
    if (r != kInsideE) return r;
  }
  dz = fabs(fabs(p.z - t->btubeOffset) - 0.5 * (t->z[t->nz - 1] - t->z[0]));
  if (dz < kTolerance) return kSurfaceE;
  return kInsideE;
}

/* ScalarDistanceToInKernel (PolyhedronImplementation.h:703-751) */
static double polyhedron_dist_in(const or_polyhedron *t, v3 p, v3 d)
{
  const int nseg = t->nz - 1;
  double tubeDistance = 0., distance = kInfLength;
  int zi;
  const v3 bp = v3_make(p.x, p.y, p.z - t->btubeOffset);
  if ((p.z < t->z[0] + kTolerance) && d.z <= 0) return kInfLength;
  if ((p.z > t->z[nseg] - kTolerance) && d.z >= 0) return kInfLength;
  if (polyhedron_inside(t, p) == kInsideE) return -1.;
  if (!tube_contains(&t->btube, bp)) {
    tubeDistance = tube_dist_in(&t->btube, bp, d);
    if (tubeDistance == kInfLength) return kInfLength;
  }
  zi = phd_clamp_z(t, phd_find_z(t, p.z));
  if (d.z >= 0) {
    for (; zi < nseg; ++zi) {
      distance = phd_dist_in_seg(t, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = phd_dist_in_seg(t, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  }
  phd_dist_endcaps(t, 0, p, d, &distance);
  return (distance >= tubeDistance - 1E-6) ? distance : kInfLength;
}

/* ScalarDistanceToOutKernel (PolyhedronImplementation.h:868-914) */
static double polyhedron_dist_out(const or_polyhedron *t, v3 p, v3 d)
{
  const int nseg = t->nz - 1;
  double distance = kInfLength;
  int zi;
  if ((p.z < t->z[0] - kTolerance) || (p.z > t->z[nseg] + kTolerance)) return -1.;
  if (polyhedron_inside(t, p) == kOutsideE) return -1.;
  zi = phd_clamp_z(t, phd_find_z(t, p.z));
  if (d.z >= 0) {
    for (; zi < nseg; ++zi) {
      distance = phd_dist_out_seg(t, zi, t->z[zi], t->z[zi + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (t->z[zi] - p.z > distance) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = phd_dist_out_seg(t, zi, t->z[zi], t->z[zi + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (p.z - t->z[zi] > distance) break;
    }
  }
  phd_dist_endcaps(t, 1, p, d, &distance);
  if (distance >= kInfLength) distance = 0.;
  return distance;
}

/* ScalarSafetyKernel (PolyhedronImplementation.h:753-800) */
static double polyhedron_safety(const or_polyhedron *t, v3 p, int pt_inside)
{
  const int nseg = t->nz - 1;
  double safety  = kInfLength, dz, s;
  int z, inside;
  const int zi = phd_clamp_z(t, phd_find_z(t, p.z));
  int phiIndex = phd_find_phi(t, p);
  inside       = phd_inside_seg_phi(t, p, zi, phiIndex);
  if (inside == kSurfaceE) return 0.;
  if ((inside == kInsideE) ^ (pt_inside != 0)) return -1.;
  for (z = zi; z < nseg;) {
    s      = phd_safety_seg2(t, z, &phiIndex, p, pt_inside);
    safety = safety < s ? safety : s;
    ++z;
    dz = t->z[z] - p.z;
    if (dz * dz > safety) break;
  }
  for (z = zi - 1; z >= 0; --z) {
    s      = phd_safety_seg2(t, z, &phiIndex, p, pt_inside);
    safety = safety < s ? safety : s;
    dz     = p.z - t->z[z];
    if (dz * dz > safety) break;
  }
  phd_safety_endcaps2(t, p, &safety);
  return sqrt(safety);
}

/* UnplacedPolyhedron::Extent (source/UnplacedPolyhedron.cpp:273-303) */
static void polyhedron_extent(const or_polyhedron *t, v3 *mn, v3 *mx)
{
  const double sidePhi = t->phiDelta / t->sides, conv = 1. / cos(0.5 * sidePhi);
  double a[3] = {kInfLength, kInfLength, kInfLength}, b[3] = {-kInfLength, -kInfLength, -kInfLength};
  int iphi, iz, k, w;
  for (iphi = 0; iphi <= t->sides; ++iphi) {
    const double phi = t->phiStart + iphi * sidePhi;
    const double cx = conv * cos(phi), cy = conv * sin(phi);
    for (iz = 0; iz < t->nz; ++iz)
      for (w = 0; w < 2; ++w) {
        const double r   = w == 0 ? t->rmin[iz] : t->rmax[iz];
        const double c[3] = {r * cx, r * cy, t->z[iz]};
        for (k = 0; k < 3; ++k) {
          a[k] = or_min(a[k], c[k]);
          b[k] = or_max(b[k], c[k]);
        }
      }
  }
  *mn = v3_make(a[0], a[1], a[2]);
  *mx = v3_make(b[0], b[1], b[2]);
}

/* ================================================================== */
/* Torus2: TorusStruct2.h, kernel/TorusImplementation2.h              */
/* ================================================================== */

/* Elementary functions of the torus' cubic solver, written out so that this restatement and
 * the GPU kernels evaluate them with the same IEEE operations (+, -, *, /, sqrt): the reference
 * calls the C library's cbrt, pow, cos and atan2, which round differently from CUDA's.  Each is
 * within a few units in the last place of the exact value; the oracle therefore equals the
 * reference build to about 1e-15 relative in the cubic's root, not bit for bit. */

/* cube root of a >= 0: a = m 2^(3q), m in [0.5, 4); Newton's iteration y <- (2 y + m / y^2) / 3
 * from a linear start, six steps (quadratic convergence from 15 % error) */
static double tor_cbrt(double a)
{
  int e, r, k;
  double m, y;
  if (a == 0.0 || !(a < kInfLength)) return a;
  m = frexp(a, &e);
  r = e % 3;
  if (r < 0) r += 3;
  m = ldexp(m, r);
  e -= r;
  y = 0.6 + 0.25 * m;
  for (k = 0; k < 6; ++k) y = (2.0 * y + m / (y * y)) / 3.0;
  return ldexp(y, e / 3);
}

/* a^(1/6) for a >= 0 */
static double tor_pow16(double a) { return sqrt(tor_cbrt(a)); }

/* atan(z), 0 <= z <= 1: two argument halvings atan(z) = 2 atan(z / (1 + sqrt(1 + z^2))) bring
 * z below tan(pi / 16), then the Taylor series to z^23 */
static double tor_atan_unit(double z)
{
  double z2, term, s;
  int k;
  z    = z / (1.0 + sqrt(1.0 + z * z));
  z    = z / (1.0 + sqrt(1.0 + z * z));
  z2   = z * z;
  term = z;
  s    = z;
  for (k = 1; k < 12; ++k) {
    term *= -z2;
    s += term / (2 * k + 1);
  }
  return 4.0 * s;
}

/* atan2(y, x) for y > 0 (the cubic solver's u) */
static double tor_atan2(double y, double x)
{
  const double ax = fabs(x);
  const double a  = (y <= ax) ? tor_atan_unit(y / ax) : 0.5 * kPi - tor_atan_unit(ax / y);
  return x < 0 ? kPi - a : a;
}

/* cos(w), |w| <= 1.1: the Taylor series to w^24 */
static double tor_cos(double w)
{
  const double w2 = w * w;
  double term = 1.0, s = 1.0;
  int k;
  for (k = 1; k <= 12; ++k) {
    term *= -w2 / ((2 * k - 1) * (2 * k));
    s += term;
  }
  return s;
}

/* SolveCubic (TorusImplementation2.h:17-53) */
static unsigned tor_solve_cubic(double a, double b, double c, double *x)
{
  const double ott = 1. / 3., sq3 = sqrt(3.), inv6sq3 = 1. / (6. * sq3);
  unsigned ireal = 1;
  const double p = b - a * a * ott;
  const double q = c - a * b * ott + 2. * a * a * a * ott * ott * ott;
  double delta   = 4 * p * p * p + 27. * q * q;
  double t, u;
  if (delta >= 0) {
    delta = sqrt(delta);
    t     = (-3 * q * sq3 + delta) * inv6sq3;
    u     = (3 * q * sq3 + delta) * inv6sq3;
    x[0]  = copysign(1., t) * tor_cbrt(fabs(t)) - copysign(1., u) * tor_cbrt(fabs(u)) - a * ott;
  } else {
    delta = sqrt(-delta);
    t     = -0.5 * q;
    u     = delta * inv6sq3;
    x[0]  = 2. * tor_pow16(t * t + u * u) * tor_cos(ott * tor_atan2(u, t));
    x[0] -= a * ott;
  }
  t     = x[0] * x[0] + a * x[0] + b;
  u     = a + x[0];
  delta = u * u - 4. * t;
  if (delta >= 0) {
    ireal = 3;
    delta = sqrt(delta);
    x[1]  = 0.5 * (-u - delta);
    x[2]  = 0.5 * (-u + delta);
  }
  return ireal;
}

static inline void tor_cmp_swap(double *v, int i, int j) /* CmpAndSwap (TorusImplementation2.h:55-66) */
{
  if (v[i] > v[j]) {
    const double c = v[j];
    v[j]           = v[i];
    v[i]           = c;
  }
}

static void tor_sort4(double *v) /* Sort4 (TorusImplementation2.h:68-77) */
{
  tor_cmp_swap(v, 0, 2);
  tor_cmp_swap(v, 1, 3);
  tor_cmp_swap(v, 0, 1);
  tor_cmp_swap(v, 2, 3);
  tor_cmp_swap(v, 1, 2);
}

/* SolveQuartic (TorusImplementation2.h:79-150) */
static int tor_solve_quartic(double a, double b, double c, double d, double *x)
{
  const double e = b - 3. * a * a / 8.;
  const double f = c + a * a * a / 8. - 0.5 * a * b;
  const double g = d - 3. * a * a * a * a / 256. + a * a * b / 16. - a * c / 4.;
  double xx[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  double delta, h = 0., j;
  unsigned ireal = 0, i;
  if (fabs(f) < 1E-6) {
    delta = e * e - 4. * g;
    if (delta < 0.) return 0;
    delta = sqrt(delta);
    h     = 0.5 * (-e - delta);
    if (h >= 0) {
      h          = sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    h = 0.5 * (-e + delta);
    if (h >= 0) {
      h          = sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    tor_sort4(x);
    return (int)ireal;
  }
  if (fabs(g) < 1E-6) {
    unsigned ncubic;
    x[ireal++] = -0.25 * a;
    ncubic     = tor_solve_cubic(0, e, f, xx);
    for (i = 0; i < ncubic; i++) x[ireal++] = xx[i] - 0.25 * a;
    tor_sort4(x);
    return (int)ireal;
  }
  ireal = tor_solve_cubic(2. * e, e * e - 4. * g, -f * f, xx);
  if (ireal == 1) {
    if (xx[0] <= 0) return 0;
    h = sqrt(xx[0]);
  } else {
    for (i = 0; i < 3; i++) {
      h = xx[i];
      if (h >= 0) break;
    }
    if (h <= 0) return 0;
    h = sqrt(h);
  }
  j     = 0.5 * (e + h * h - f / h);
  ireal = 0;
  delta = h * h - 4. * j;
  if (delta >= 0) {
    delta      = sqrt(delta);
    x[ireal++] = 0.5 * (-h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (-h + delta) - 0.25 * a;
  }
  delta = h * h - 4. * g / j;
  if (delta >= 0) {
    delta      = sqrt(delta);
    x[ireal++] = 0.5 * (h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (h + delta) - 0.25 * a;
  }
  tor_sort4(x);
  return (int)ireal;
}

/* TorusStruct2(rmin, rmax, rtor, sphi, dphi) (TorusStruct2.h:36-43); the bounding tube
 * GenericUnplacedTube(rtor - rmax - tol, rtor + rmax + tol, rmax, sphi, dphi) */
static int torus_init(or_torus *t, const double *a, char *err, int errlen)
{
  double tp[5];
  t->rmin = a[0];
  t->rmax = a[1];
  t->rtor = a[2];
  t->sphi = a[3];
  t->dphi = a[4];
  if (!(t->rmin >= 0 && t->rmax > t->rmin && t->rtor > t->rmax + kTolerance && t->dphi > 0)) {
    set_err(err, errlen, "torus: needs 0 <= rmin < rmax < rtor and dphi > 0");
    return -1;
  }
  t->rmin2 = t->rmin * t->rmin;
  t->rmax2 = t->rmax * t->rmax;
  t->rtor2 = t->rtor * t->rtor;
  wedge_init(&t->w, t->dphi, t->sphi);
  tp[0] = t->rtor - t->rmax - kTolerance;
  tp[1] = t->rtor + t->rmax + kTolerance;
  tp[2] = t->rmax;
  tp[3] = t->sphi;
  tp[4] = t->dphi;
  return tube_init(&t->btube, tp, err, errlen);
}

static inline int torus_has_phi(const or_torus *t) { return t->dphi < kTwoPi; }

/* GenericKernelForContainsAndInside<ForInside, notForDisk> (TorusImplementation2.h:241-285) */
static void torus_ci(const or_torus *t, v3 p, int forInside, int notForDisk, int *cin, int *cout)
{
  const double tol   = 100. * kTolerance;
  const double rxy   = sqrt(p.x * p.x + p.y * p.y);
  const double radsq = (rxy - t->rtor) * (rxy - t->rtor) + p.z * p.z;
  if (forInside) {
    *cout = radsq > (tol * t->rmax + t->rmax2);
    *cin  = radsq < (-tol * t->rmax + t->rmax2);
  } else {
    *cout = radsq > t->rmax2;
  }
  if (*cout) return;
  if (forInside) {
    *cout |= radsq < (-tol * t->rmin + t->rmin2);
    *cin &= radsq > (tol * t->rmin + t->rmin2);
  } else {
    *cout |= radsq < t->rmin2;
  }
  if (*cout) return;
  if (torus_has_phi(t) && notForDisk) {
    int cinphi = 0, coutphi = 0;
    wedge_ci(&t->w, p, forInside, &cinphi, &coutphi);
    *cout |= coutphi;
    if (forInside) *cin &= cinphi;
  }
}

/* Contains (TorusImplementation2.h:391-399): the inside tolerances and no phi test, as the
 * reference has it */
static int torus_contains(const or_torus *t, v3 p)
{
  int cin = 0, cout = 0;
  torus_ci(t, p, 1, 0, &cin, &cout);
  return !cout;
}

static int torus_inside(const or_torus *t, v3 p) /* InsideKernel (TorusImplementation2.h:227-239) */
{
  int cin = 0, cout = 0;
  torus_ci(t, p, 1, 1, &cin, &cout);
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

static int torus_contains_disk(const or_torus *t, v3 p) /* UnplacedContainsDisk (TorusImplementation2.h:219-225) */
{
  int cin = 0, cout = 0;
  torus_ci(t, p, 0, 0, &cin, &cout);
  return !cout;
}

/* ToBoundary<ForRmin> (TorusImplementation2.h:287-377) */
static double torus_to_boundary(const or_torus *t, v3 pt, v3 dir, double radius, int out)
{
  const double tol = 100. * kTolerance;
  const double r0sq   = pt.x * pt.x + pt.y * pt.y + pt.z * pt.z;
  const double rdotn  = pt.x * dir.x + pt.y * dir.y + pt.z * dir.z;
  const double rsumsq = t->rtor2 + radius * radius;
  const double a      = 4. * rdotn;
  const double b      = 2. * (r0sq + 2. * rdotn * rdotn - rsumsq + 2. * t->rtor2 * dir.z * dir.z);
  const double c      = 4. * (r0sq * rdotn - rsumsq * rdotn + 2. * t->rtor2 * pt.z * dir.z);
  const double d = r0sq * r0sq - 2. * r0sq * rsumsq + 4. * t->rtor2 * pt.z * pt.z +
                   (t->rtor2 - radius * radius) * (t->rtor2 - radius * radius);
  double x[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  int nsol = 0, inner, i;
  if (fabs(dir.z) < 1E-3 && fabs(pt.z) < 0.1 * radius) {
    double r0            = t->rtor - sqrt((radius - pt.z) * (radius + pt.z));
    const double invdxy2 = 1. / (1 - dir.z * dir.z);
    const double b0      = (pt.x * dir.x + pt.y * dir.y) * invdxy2;
    double c0            = (pt.x * pt.x + (pt.y - r0) * (pt.y + r0)) * invdxy2;
    double delta         = b0 * b0 - c0;
    if (delta > 0) {
      x[nsol] = -b0 - sqrt(delta);
      if (x[nsol] > -tol) nsol++;
      x[nsol] = -b0 + sqrt(delta);
      if (x[nsol] > -tol) nsol++;
    }
    r0    = t->rtor + sqrt((radius - pt.z) * (radius + pt.z));
    c0    = (pt.x * pt.x + (pt.y - r0) * (pt.y + r0)) * invdxy2;
    delta = b0 * b0 - c0;
    if (delta > 0) {
      x[nsol] = -b0 - sqrt(delta);
      if (x[nsol] > -tol) nsol++;
      x[nsol] = -b0 + sqrt(delta);
      if (x[nsol] > -tol) nsol++;
    }
    if (nsol) tor_sort4(x);
  } else {
    nsol = tor_solve_quartic(a, b, c, d, x);
  }
  if (!nsol) return kInfLength;
  inner = fabs(radius - t->rmin) < kTolerance;
  for (i = 0; i < nsol; i++) {
    v3 r0, norm;
    double ndotd, s, eps, delta, eps0, inv;
    int ntry;
    if (x[i] < -10) continue;
    r0   = v3_add(pt, v3_scale(x[i], dir));
    norm = r0;
    r0.z = 0.;
    inv  = 1. / sqrt(v3_mag2(r0));
    r0   = v3_make(r0.x * inv, r0.y * inv, r0.z * inv);
    r0   = v3_make(r0.x * t->rtor, r0.y * t->rtor, r0.z * t->rtor);
    norm = v3_sub(norm, r0);
    ndotd = v3_dot(norm, dir);
    if (inner ^ out) {
      if (ndotd < 0) continue;
    } else {
      if (ndotd > 0) continue;
    }
    if (torus_has_phi(t)) {
      int cin = 0, cout = 0;
      wedge_ci(&t->w, r0, 1, &cin, &cout); /* Wedge::ContainsWithBoundary */
      if (cout) continue;
    }
    s     = x[i];
    eps   = kInfLength;
    delta = s * s * s * s + a * s * s * s + b * s * s + c * s + d;
    eps0  = -delta / (4. * s * s * s + 3. * a * s * s + 2. * b * s + c);
    ntry  = 0;
    while (fabs(eps) > kTolerance) {
      if (fabs(eps0) > 100) break;
      s += eps0;
      if (fabs(s + eps0) < kTolerance) break;
      delta = s * s * s * s + a * s * s * s + b * s * s + c * s + d;
      eps   = -delta / (4. * s * s * s + 3. * a * s * s + 2. * b * s + c);
      if (fabs(eps) >= fabs(eps0)) break;
      ntry++;
      if (ntry > 100) break;
      eps0 = eps;
    }
    if (s < -tol) continue;
    return 0. > s ? 0. : s;
  }
  return kInfLength;
}

/* DistSqrToTorusR (TorusImplementation2.h:149-156) */
static double torus_dist2_axis(const or_torus *t, v3 p, v3 dir, double dist)
{
  const v3 q       = v3_add(p, v3_scale(dist, dir));
  const double rxy = sqrt(q.x * q.x + q.y * q.y);
  return (rxy - t->rtor) * (rxy - t->rtor) + q.z * q.z;
}

/* DistanceToIn (TorusImplementation2.h:415-491), the VECGEOM_NO_SPECIALIZATION branch */
static double torus_dist_in(const or_torus *t, v3 p, v3 d)
{
  double distance = kInfLength, tubeDistance = kInfLength, dd;
  v3 lp = p;
  const int inBounds = tube_contains(&t->btube, lp);
  if (!inBounds)
    tubeDistance = tube_dist_in(&t->btube, lp, d);
  else
    tubeDistance = 0.;
  if (inBounds) {
    if (torus_inside(t, p) == kInsideE) return -1.;
  } else if (tubeDistance == kInfLength) {
    return kInfLength;
  }
  lp = v3_add(lp, v3_scale(tubeDistance, d));
  if (torus_has_phi(t)) {
    double d1, d2;
    wedge_dist(&t->w, lp, d, 1, &d1, &d2);
    if (d1 != kInfLength) {
      const double daxis = torus_dist2_axis(t, lp, d, d1);
      if (daxis >= t->rmin2 && daxis < t->rmax2) {
        distance = d1;
        if (fabs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    if (d2 != kInfLength) {
      const double daxis = torus_dist2_axis(t, lp, d, d2);
      if (daxis >= t->rmin2 && daxis < t->rmax2) {
        distance = d2 < distance ? d2 : distance;
        if (fabs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    distance = kInfLength;
  }
  dd = torus_to_boundary(t, lp, d, t->rmax, 0);
  if (t->rmin > 0.) {
    const double ddrmin = torus_to_boundary(t, lp, d, t->rmin, 0);
    dd                  = dd < ddrmin ? dd : ddrmin;
  }
  distance = distance < dd ? distance : dd;
  distance += tubeDistance;
  if (fabs(distance) > kInfLength) distance = kInfLength;
  return distance;
}

/* DistanceToOut (TorusImplementation2.h:158-217) */
static double torus_dist_out(const or_torus *t, v3 p, v3 d)
{
  const double rsq = p.x * p.x + p.y * p.y;
  const double outerExcl = t->rtor + t->rmax + kHalfTolerance, innerExcl = t->rtor - t->rmax - kHalfTolerance;
  double distance, dout, din = kInfLength;
  if (fabs(p.z) - t->rmax > kHalfTolerance || rsq > outerExcl * outerExcl || rsq < innerExcl * innerExcl) return -1.;
  if (torus_inside(t, p) == kOutsideE) return -1.;
  dout = torus_to_boundary(t, p, d, t->rmax, 1);
  if (t->rmin > 0) din = torus_to_boundary(t, p, d, t->rmin, 1);
  distance = dout < din ? dout : din;
  if (torus_has_phi(t)) {
    double dp1, dp2;
    wedge_dist(&t->w, p, d, 0, &dp1, &dp2);
    if (dp1 < distance) {
      const v3 ip = v3_add(p, v3_scale(dp1, d));
      if (torus_contains_disk(t, ip)) {
        const double diri = ip.x * t->w.a1x + ip.y * t->w.a1y;
        if (diri >= 0) distance = dp1;
      }
    }
    if (dp2 < distance) {
      const v3 ip = v3_add(p, v3_scale(dp2, d));
      if (torus_contains_disk(t, ip)) {
        const double diri2 = ip.x * t->w.a2x + ip.y * t->w.a2y;
        if (diri2 >= 0 && dp2 < distance) distance = dp2;
      }
    }
  }
  if (distance >= kInfLength) distance = -1.;
  return distance;
}

/* SafetyToIn (TorusImplementation2.h:493-509) */
static double torus_safe_in(const or_torus *t, v3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t->rtor) * (rxy - t->rtor) + p.z * p.z);
  double safety    = rad - t->rmax;
  if (t->rmin) safety = or_max(t->rmin - rad, rad - t->rmax);
  if (torus_has_phi(t) && rxy != 0.) safety = or_max(wedge_safe_in(&t->w, p), safety);
  return safety;
}

/* SafetyToOut (TorusImplementation2.h:379-389) */
static double torus_safe_out(const or_torus *t, v3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t->rtor) * (rxy - t->rtor) + p.z * p.z);
  double safety    = t->rmax - rad;
  if (t->rmin) safety = or_min(rad - t->rmin, t->rmax - rad);
  if (torus_has_phi(t)) safety = or_min(wedge_safe_out(&t->w, p), safety);
  return safety;
}

/* ---------------------------------------------------------------- */
/* Boolean solids over placed operands: BooleanImplementation.h (subtraction),
 * BooleanUnionImplementation.h, BooleanIntersectionImplementation.h.  A placed operand's
 * Contains, Inside, DistanceToIn, PlacedDistanceToOut and SafetyToIn take the boolean-frame
 * point into the operand's frame (SpecializedPlacedVolImplHelper.h:99-172); its DistanceToOut
 * and SafetyToOut do not (PlacedVolImplHelper.h:76-100).  The reference's loops are unbounded;
 * these stop after OR_BOOL_MAX_ITER rounds (never reached on a valid solid). */
#define OR_BOOL_MAX_ITER 1000000
enum { OR_INSIDE = 1, OR_SURFACE = 2, OR_OUTSIDE = 3 };

static int bo_contains(const or_lv *o, const or_xf *x, v3 p, or_counters *c)
{
  return shape_contains(o, xf_transform(x, p), c);
}
static int bo_inside(const or_lv *o, const or_xf *x, v3 p, or_counters *c)
{
  return shape_inside(o, xf_transform(x, p), c);
}
static double bo_dist_in(const or_lv *o, const or_xf *x, v3 p, v3 d, double stepmax, or_counters *c)
{
  return shape_dist_in(o, xf_transform(x, p), xf_transform_dir(x, d), stepmax, c);
}
static double bo_placed_dist_out(const or_lv *o, const or_xf *x, v3 p, v3 d, double stepmax, or_counters *c)
{
  return shape_dist_out(o, xf_transform(x, p), xf_transform_dir(x, d), stepmax, c);
}
static double bo_safe_in(const or_lv *o, const or_xf *x, v3 p, or_counters *c)
{
  return shape_safe_in(o, xf_transform(x, p), c);
}
static v3 v3_axpy(v3 p, double a, v3 d) { return v3_make(p.x + a * d.x, p.y + a * d.y, p.z + a * d.z); }

static int boolean_contains(const or_boolean *b, v3 p, or_counters *c)
{
  switch (b->op) {
  case 0: /* BooleanUnionImplementation.h Contains */
    if (bo_contains(b->left, &b->lxf, p, c)) return 1;
    return bo_contains(b->right, &b->rxf, p, c);
  case 1: /* BooleanIntersectionImplementation.h Contains */
  {
    const int a = bo_contains(b->left, &b->lxf, p, c);
    const int r = bo_contains(b->right, &b->rxf, p, c);
    return a && r;
  }
  default: /* BooleanImplementation.h Contains (subtraction) */
    if (!bo_contains(b->left, &b->lxf, p, c)) return 0;
    return !bo_contains(b->right, &b->rxf, p, c);
  }
}

/* -1: a union point on both operands' surfaces, whose answer takes their normals (unsupported) */
static int boolean_inside(const or_boolean *b, v3 p, or_counters *c)
{
  const int a = bo_inside(b->left, &b->lxf, p, c);
  int r;
  switch (b->op) {
  case 0:
    if (a == OR_INSIDE) return OR_INSIDE;
    r = bo_inside(b->right, &b->rxf, p, c);
    if (r == OR_INSIDE) return OR_INSIDE;
    if (a == OR_SURFACE && r == OR_SURFACE) return -1;
    if (r == OR_SURFACE || a == OR_SURFACE) return OR_SURFACE;
    return OR_OUTSIDE;
  case 1:
    if (a == OR_OUTSIDE) return OR_OUTSIDE;
    r = bo_inside(b->right, &b->rxf, p, c);
    if (a == OR_INSIDE && r == OR_INSIDE) return OR_INSIDE;
    if ((a == OR_INSIDE && r == OR_SURFACE) || (r == OR_INSIDE && a == OR_SURFACE) ||
        (a == OR_SURFACE && r == OR_SURFACE))
      return OR_SURFACE;
    return OR_OUTSIDE;
  default:
    if (a == OR_OUTSIDE) return OR_OUTSIDE;
    r = bo_inside(b->right, &b->rxf, p, c);
    if (a == OR_INSIDE && r == OR_OUTSIDE) return OR_INSIDE;
    if ((a == OR_INSIDE && r == OR_SURFACE) || (r == OR_OUTSIDE && a == OR_SURFACE)) return OR_SURFACE;
    return OR_OUTSIDE;
  }
}

static double boolean_dist_in(const or_boolean *b, v3 p, v3 d, double stepmax, or_counters *c)
{
  const or_lv *L = b->left, *R = b->right;
  const or_xf *lx = &b->lxf, *rx = &b->rxf;
  long it;
  if (b->op == 0) { /* union */
    const double d1 = bo_dist_in(L, lx, p, d, stepmax, c);
    const double d2 = bo_dist_in(R, rx, p, d, stepmax, c);
    return d1 < d2 ? d1 : d2; /* Min */
  }
  if (b->op == 1) { /* intersection */
    v3 hit      = p;
    int inleft  = bo_contains(L, lx, hit, c);
    int inright = bo_contains(R, rx, hit, c);
    double d1 = 0., d2 = 0., snext = 0.;
    if (inleft && inright) {
      d1 = bo_placed_dist_out(L, lx, hit, d, stepmax, c);
      d2 = bo_placed_dist_out(R, rx, hit, d, stepmax, c);
      if (d1 < 2 * kTolerance) inleft = 0;
      if (d2 < 2 * kTolerance) inright = 0;
      if (inleft && inright) return 0.0;
    }
    for (it = 0; it < OR_BOOL_MAX_ITER; ++it) {
      d1 = d2 = 0;
      if (!inleft) {
        d1 = bo_dist_in(L, lx, hit, d, kInfLength, c);
        d1 = d1 > kTolerance ? d1 : kTolerance; /* Max */
        if (d1 > 1E20) return kInfLength;
      }
      if (!inright) {
        d2 = bo_dist_in(R, rx, hit, d, kInfLength, c);
        d2 = d2 > kTolerance ? d2 : kTolerance;
        if (d2 > 1E20) return kInfLength;
      }
      if (d1 > d2) {
        snext += d1;
        inleft  = 1;
        hit     = v3_axpy(hit, d1, d);
        inright = bo_contains(R, rx, v3_axpy(hit, kTolerance, d), c);
        if (inright) return snext;
      } else {
        snext += d2;
        inright = 1;
        hit     = v3_axpy(hit, d2, d);
        inleft  = bo_contains(L, lx, v3_axpy(hit, kTolerance, d), c);
        if (inleft) return snext;
      }
    }
    return kInfLength;
  }
  { /* subtraction */
    double d1, d2, snxt = 0.;
    v3 hit              = p;
    int insideRight     = bo_contains(R, rx, p, c);
    const double epsil  = kPushTolerance;
    for (it = 0; it < OR_BOOL_MAX_ITER; ++it) {
      if (insideRight) {
        d1 = bo_placed_dist_out(R, rx, hit, d, stepmax, c);
        snxt += (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : 0.;
        hit = v3_axpy(hit, (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : 0., d);
        if (bo_contains(L, lx, hit, c)) {
          const double check = bo_placed_dist_out(L, lx, hit, d, kInfLength, c);
          if (check > epsil) return snxt;
        }
      }
      d2 = bo_dist_in(L, lx, hit, d, stepmax, c);
      d2 = d2 > 0. ? d2 : 0.; /* Max(d2, 0) */
      if (d2 == kInfLength) return kInfLength;
      d1 = bo_dist_in(R, rx, hit, d, stepmax, c);
      if (d2 < d1 - kTolerance) {
        snxt += d2 + epsil;
        return snxt;
      }
      snxt += (d1 >= 0. && d1 < kInfLength) ? d1 + epsil : 0.;
      hit         = v3_axpy(hit, (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : epsil, d);
      insideRight = 1;
    }
    return kInfLength;
  }
}

/* BooleanUnionImplementation.h DistanceToOut: the loop over connecting operands */
static double union_dist_out_walk(const or_lv *A, const or_xf *ax, const or_lv *B, const or_xf *bx, v3 p, v3 d,
                                  or_counters *c)
{
  double dist = 0.;
  const double pushdist = kPushTolerance;
  v3 nextp = p;
  int connecting;
  long it = 0;
  do {
    double disTmp;
    connecting = 0;
    disTmp     = bo_placed_dist_out(A, ax, nextp, d, kInfLength, c);
    dist += (disTmp >= 0. && disTmp < kInfLength) ? disTmp : 0;
    dist += pushdist;
    nextp = v3_axpy(p, dist, d);
    if (bo_inside(B, bx, nextp, c) != OR_OUTSIDE) {
      disTmp = bo_placed_dist_out(B, bx, nextp, d, kInfLength, c);
      dist += (disTmp >= 0. && disTmp < kInfLength) ? disTmp : 0;
      dist += pushdist;
      nextp      = v3_axpy(p, dist, d);
      connecting = 1;
    }
  } while (connecting && bo_inside(A, ax, nextp, c) != OR_OUTSIDE && ++it < OR_BOOL_MAX_ITER);
  return dist;
}

static double boolean_dist_out(const or_boolean *b, v3 p, v3 d, double stepmax, or_counters *c)
{
  const or_lv *L = b->left, *R = b->right;
  const or_xf *lx = &b->lxf, *rx = &b->rxf;
  if (b->op == 0) {
    const int posA = bo_inside(L, lx, p, c);
    const double dist = posA != OR_OUTSIDE ? union_dist_out_walk(L, lx, R, rx, p, d, c)
                                           : union_dist_out_walk(R, rx, L, lx, p, d, c);
    double distance = dist - kPushTolerance;
    if (distance < kTolerance && posA == OR_OUTSIDE && bo_inside(R, rx, p, c) == OR_OUTSIDE) distance = -kTolerance;
    return distance;
  }
  if (b->op == 1) {
    const double a = shape_dist_out(L, p, d, kInfLength, c); /* the left operand unplaced */
    const double r = bo_placed_dist_out(R, rx, p, d, kInfLength, c);
    return a < r ? a : r;
  }
  {
    const double distancel = bo_placed_dist_out(L, lx, p, d, stepmax, c);
    const double dinright  = bo_dist_in(R, rx, p, d, stepmax, c);
    return distancel < dinright ? distancel : dinright;
  }
}

static double boolean_safe_in(const or_boolean *b, v3 p, or_counters *c)
{
  const or_lv *L = b->left, *R = b->right;
  const or_xf *lx = &b->lxf, *rx = &b->rxf;
  if (b->op == 0) {
    const double a = bo_safe_in(L, lx, p, c), r = bo_safe_in(R, rx, p, c);
    return a < r ? a : r;
  }
  if (b->op == 1) {
    const int insideA = bo_contains(L, lx, p, c);
    const int insideB = bo_contains(R, rx, p, c);
    if (!insideA && insideB) return bo_safe_in(L, lx, p, c);
    if (!insideB && insideA) return bo_safe_in(R, rx, p, c);
    {
      const double a = bo_safe_in(L, lx, p, c), r = bo_safe_in(R, rx, p, c);
      return a < r ? a : r;
    }
  }
  if (bo_contains(L, lx, p, c) && bo_contains(R, rx, p, c)) return shape_safe_out(R, xf_transform(rx, p), c);
  return bo_safe_in(L, lx, p, c);
}

static double boolean_safe_out(const or_boolean *b, v3 p, or_counters *c)
{
  const or_lv *L = b->left, *R = b->right;
  const or_xf *lx = &b->lxf, *rx = &b->rxf;
  if (b->op == 0) {
    const int insideA = bo_inside(L, lx, p, c);
    const int insideB = bo_inside(R, rx, p, c);
    if (insideA == OR_OUTSIDE && insideB == OR_OUTSIDE) return -kTolerance;
    if (insideA != OR_OUTSIDE && insideB != OR_OUTSIDE) {
      const double a = shape_safe_out(L, p, c), r = shape_safe_out(R, xf_transform(rx, p), c);
      return a > r ? a : r; /* Max */
    }
    if (insideA == OR_SURFACE || insideB == OR_SURFACE) return -kTolerance;
    if (insideA == OR_OUTSIDE) return shape_safe_out(R, xf_transform(rx, p), c);
    return shape_safe_out(L, p, c);
  }
  if (b->op == 1) {
    const double a = shape_safe_out(L, p, c), r = shape_safe_out(R, xf_transform(rx, p), c);
    double safety = a < r ? a : r;
    if (safety < 0.) safety = 0.;
    return safety;
  }
  {
    const double a = shape_safe_out(L, p, c), r = bo_safe_in(R, rx, p, c);
    return a < r ? a : r;
  }
}

/* VPlacedVolume::Extent (source/PlacedVolume.cpp:139-175): the shape's extent taken into its
 * mother's frame (the eight corners when the placement rotates, else the two extremes) */
static void placed_extent(const or_lv *o, const or_xf *x, v3 *mn, v3 *mx)
{
  v3 pmin, pmax;
  shape_extent(o, &pmin, &pmax);
  if (x->has_rot) {
    v3 b[8];
    int i;
    b[0] = xf_inverse_transform(x, v3_make(pmin.x, pmin.y, pmin.z));
    b[1] = xf_inverse_transform(x, v3_make(pmax.x, pmin.y, pmin.z));
    b[2] = xf_inverse_transform(x, v3_make(pmin.x, pmax.y, pmin.z));
    b[3] = xf_inverse_transform(x, v3_make(pmax.x, pmax.y, pmin.z));
    b[4] = xf_inverse_transform(x, v3_make(pmin.x, pmin.y, pmax.z));
    b[5] = xf_inverse_transform(x, v3_make(pmax.x, pmin.y, pmax.z));
    b[6] = xf_inverse_transform(x, v3_make(pmin.x, pmax.y, pmax.z));
    b[7] = xf_inverse_transform(x, v3_make(pmax.x, pmax.y, pmax.z));
    *mn = b[0];
    *mx = b[0];
    for (i = 1; i < 8; ++i) {
      *mn = v3_make(or_min(mn->x, b[i].x), or_min(mn->y, b[i].y), or_min(mn->z, b[i].z));
      *mx = v3_make(or_max(mx->x, b[i].x), or_max(mx->y, b[i].y), or_max(mx->z, b[i].z));
    }
  } else {
    *mn = xf_inverse_transform(x, pmin);
    *mx = xf_inverse_transform(x, pmax);
  }
}

/* TransformedExtent (source/UnplacedBooleanVolume.cpp:403-442): the box of the operand's
 * placed extent, whose corners it takes through the placement once more (the placed extent is
 * already in the boolean's frame, so a translated or rotated operand's box comes out larger
 * than the operand; the reference's extents, and so its bounding boxes, are these) */
static void transformed_extent(const or_lv *o, const or_xf *x, v3 *mn, v3 *mx)
{
  v3 lower, upper, delta;
  double minx = kInfLength, miny = kInfLength, minz = kInfLength;
  double maxx = -kInfLength, maxy = -kInfLength, maxz = -kInfLength;
  int i, j, k;
  placed_extent(o, x, &lower, &upper);
  delta = v3_sub(upper, lower);
  for (i = 0; i <= 1; ++i)
    for (j = 0; j <= 1; ++j)
      for (k = 0; k <= 1; ++k) {
        v3 corner, tc;
        corner.x = lower.x + i * delta.x;
        corner.y = lower.y + j * delta.y;
        corner.z = lower.z + k * delta.z;
        tc       = xf_inverse_transform(x, corner);
        minx     = tc.x < minx ? tc.x : minx; /* std::min(minx, v) */
        miny     = tc.y < miny ? tc.y : miny;
        minz     = tc.z < minz ? tc.z : minz;
        maxx     = maxx < tc.x ? tc.x : maxx; /* std::max(maxx, v) */
        maxy     = maxy < tc.y ? tc.y : maxy;
        maxz     = maxz < tc.z ? tc.z : maxz;
      }
  *mn = v3_make(minx, miny, minz);
  *mx = v3_make(maxx, maxy, maxz);
}

/* UnplacedBooleanVolume<op>::Extent (source/UnplacedBooleanVolume.cpp:444-490) */
static void boolean_extent(const or_boolean *b, v3 *mn, v3 *mx)
{
  v3 minL, maxL, minR, maxR;
  transformed_extent(b->left, &b->lxf, &minL, &maxL);
  transformed_extent(b->right, &b->rxf, &minR, &maxR);
  if (b->op == 2) {
    *mn = minL;
    *mx = maxL;
  } else if (b->op == 0) {
    *mn = v3_make(minL.x < minR.x ? minL.x : minR.x, minL.y < minR.y ? minL.y : minR.y,
                  minL.z < minR.z ? minL.z : minR.z);
    *mx = v3_make(maxL.x > maxR.x ? maxL.x : maxR.x, maxL.y > maxR.y ? maxL.y : maxR.y,
                  maxL.z > maxR.z ? maxL.z : maxR.z);
  } else {
    *mn = v3_make(minL.x > minR.x ? minL.x : minR.x, minL.y > minR.y ? minL.y : minR.y,
                  minL.z > minR.z ? minL.z : minR.z);
    *mx = v3_make(maxL.x < maxR.x ? maxL.x : maxR.x, maxL.y < maxR.y ? maxL.y : maxR.y,
                  maxL.z < maxR.z ? maxL.z : maxR.z);
  }
}

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
  case OR_CONE: return cone_init(&lv->s.cone, p, err, errlen);
  case OR_TRD: return trd_init(&lv->s.trd, p, err, errlen);
  case OR_TRAP: return trap_init(&lv->s.trap, p, err, errlen);
  case OR_SPHERE: return sphere_init(&lv->s.sph, p, err, errlen);
  case OR_POLYCONE: return polycone_init(&lv->s.pcon, p, err, errlen);
  case OR_ORB:
    lv->s.orb.r = p[0];
    return 0;
  case OR_CUTTUBE: return cuttube_init(&lv->s.ctube, p, err, errlen);
  case OR_POLYHEDRON: return polyhedron_init(&lv->s.phd, p, err, errlen);
  case OR_TORUS: return torus_init(&lv->s.tor, p, err, errlen);
  case OR_BOOLEAN: /* operands are linked once the placements are known (or_core.c) */
    if (!(p[0] == 0. || p[0] == 1. || p[0] == 2.) || !(p[1] >= 0. && p[1] <= 2147483647. && p[1] == floor(p[1])) ||
        !(p[2] >= 0. && p[2] <= 2147483647. && p[2] == floor(p[2]))) {
      set_err(err, errlen, "boolean: bad operation or operand ids");
      return -1;
    }
    lv->s.boo.op       = (int)p[0];
    lv->s.boo.left_pv  = (int)p[1];
    lv->s.boo.right_pv = (int)p[2];
    return 0;
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
  case OR_CONE: cone_extent(&lv->s.cone, mn, mx); return;
  case OR_TRD: trd_extent(&lv->s.trd, mn, mx); return;
  case OR_TRAP: trap_extent(&lv->s.trap, mn, mx); return;
  case OR_SPHERE: sphere_extent(&lv->s.sph, mn, mx); return;
  case OR_POLYCONE: polycone_extent(&lv->s.pcon, mn, mx); return;
  case OR_ORB:
    *mn = v3_make(-lv->s.orb.r, -lv->s.orb.r, -lv->s.orb.r);
    *mx = v3_make(lv->s.orb.r, lv->s.orb.r, lv->s.orb.r);
    return;
  case OR_CUTTUBE: cuttube_extent(&lv->s.ctube, mn, mx); return;
  case OR_BOOLEAN: boolean_extent(&lv->s.boo, mn, mx); return;
  case OR_POLYHEDRON: polyhedron_extent(&lv->s.phd, mn, mx); return;
  case OR_TORUS: tube_extent(&lv->s.tor.btube, mn, mx); return; /* UnplacedTorus2.h:210 */
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
  case OR_CONE: return cone_dist_in(&lv->s.cone, p, d);
  case OR_TRD: return trd_dist_in(&lv->s.trd, p, d);
  case OR_TRAP: return trap_dist_in(&lv->s.trap, p, d);
  case OR_SPHERE: return sphere_dist_in(&lv->s.sph, p, d);
  case OR_POLYCONE: return polycone_dist_in(&lv->s.pcon, p, d);
  case OR_ORB: return orb_dist_in(&lv->s.orb, p, d);
  case OR_CUTTUBE: return cuttube_dist_in(&lv->s.ctube, p, d, stepmax);
  case OR_BOOLEAN: return boolean_dist_in(&lv->s.boo, p, d, stepmax, c);
  case OR_POLYHEDRON: return polyhedron_dist_in(&lv->s.phd, p, d);
  case OR_TORUS: return torus_dist_in(&lv->s.tor, p, d);
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
  case OR_CONE: return cone_dist_out(&lv->s.cone, p, d);
  case OR_TRD: return trd_dist_out(&lv->s.trd, p, d);
  case OR_TRAP: return trap_dist_out(&lv->s.trap, p, d);
  case OR_SPHERE: return sphere_dist_out(&lv->s.sph, p, d);
  case OR_POLYCONE: return polycone_dist_out(&lv->s.pcon, p, d);
  case OR_ORB: return orb_dist_out(&lv->s.orb, p, d);
  case OR_CUTTUBE: return cuttube_dist_out(&lv->s.ctube, p, d);
  case OR_BOOLEAN: return boolean_dist_out(&lv->s.boo, p, d, stepmax, c);
  case OR_POLYHEDRON: return polyhedron_dist_out(&lv->s.phd, p, d);
  case OR_TORUS: return torus_dist_out(&lv->s.tor, p, d);
  }
  return -1.;
}

double shape_safe_in(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_SAFE_IN);
  switch (lv->type) {
  case OR_BOX: return box_safe_in(&lv->s.box, p);
  case OR_TUBE: return tube_safe_in(&lv->s.tube, p);
  case OR_CONE: return cone_safe_in(&lv->s.cone, p);
  case OR_TRD: return trd_safety(&lv->s.trd, p, 0);
  case OR_TRAP: return trap_safe_in(&lv->s.trap, p);
  case OR_SPHERE: return sphere_safe_in(&lv->s.sph, p);
  case OR_POLYCONE: return polycone_safe_in(&lv->s.pcon, p);
  case OR_ORB: return orb_safe_in(&lv->s.orb, p);
  case OR_CUTTUBE: return cuttube_safe_in(&lv->s.ctube, p);
  case OR_BOOLEAN: return boolean_safe_in(&lv->s.boo, p, c);
  case OR_POLYHEDRON: return polyhedron_safety(&lv->s.phd, p, 0);
  case OR_TORUS: return torus_safe_in(&lv->s.tor, p);
  }
  return kInfLength;
}

double shape_safe_out(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_SAFE_OUT);
  switch (lv->type) {
  case OR_BOX: return box_safe_out(&lv->s.box, p);
  case OR_TUBE: return tube_safe_out(&lv->s.tube, p);
  case OR_CONE: return cone_safe_out(&lv->s.cone, p);
  case OR_TRD: return trd_safety(&lv->s.trd, p, 1);
  case OR_TRAP: return trap_safe_out(&lv->s.trap, p);
  case OR_SPHERE: return sphere_safe_out(&lv->s.sph, p);
  case OR_POLYCONE: return polycone_safe_out(&lv->s.pcon, p);
  case OR_ORB: return orb_safe_out(&lv->s.orb, p);
  case OR_CUTTUBE: return cuttube_safe_out(&lv->s.ctube, p);
  case OR_BOOLEAN: return boolean_safe_out(&lv->s.boo, p, c);
  case OR_POLYHEDRON: return polyhedron_safety(&lv->s.phd, p, 1);
  case OR_TORUS: return torus_safe_out(&lv->s.tor, p);
  }
  return 0.;
}

int shape_contains(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_CONTAINS);
  switch (lv->type) {
  case OR_BOX: return box_contains(&lv->s.box, p);
  case OR_TUBE: return tube_contains(&lv->s.tube, p);
  case OR_CONE: return cone_contains(&lv->s.cone, p);
  case OR_TRD: return trd_contains(&lv->s.trd, p);
  case OR_TRAP: return trap_contains(&lv->s.trap, p);
  case OR_SPHERE: return sphere_contains(&lv->s.sph, p);
  case OR_POLYCONE: return polycone_contains(&lv->s.pcon, p);
  case OR_ORB: return orb_contains(&lv->s.orb, p);
  case OR_CUTTUBE: return cuttube_contains(&lv->s.ctube, p);
  case OR_BOOLEAN: return boolean_contains(&lv->s.boo, p, c);
  case OR_POLYHEDRON: return polyhedron_contains(&lv->s.phd, p);
  case OR_TORUS: return torus_contains(&lv->s.tor, p);
  }
  return 0;
}

int shape_inside(const or_lv *lv, v3 p, or_counters *c)
{
  COUNT(OR_OP_INSIDE);
  switch (lv->type) {
  case OR_BOX: return box_inside(&lv->s.box, p);
  case OR_TUBE: return tube_inside(&lv->s.tube, p);
  case OR_CONE: return cone_inside(&lv->s.cone, p);
  case OR_TRD: return trd_inside(&lv->s.trd, p);
  case OR_TRAP: return trap_inside(&lv->s.trap, p);
  case OR_SPHERE: return sphere_inside(&lv->s.sph, p);
  case OR_POLYCONE: return polycone_inside(&lv->s.pcon, p);
  case OR_ORB: return orb_inside(&lv->s.orb, p);
  case OR_CUTTUBE: return cuttube_inside(&lv->s.ctube, p);
  case OR_BOOLEAN: return boolean_inside(&lv->s.boo, p, c);
  case OR_POLYHEDRON: return polyhedron_inside(&lv->s.phd, p);
  case OR_TORUS: return torus_inside(&lv->s.tor, p);
  }
  return kOutsideE;
}
