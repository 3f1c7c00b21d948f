// shapes_fp64.cuh -- FP64 device kernels of the unplaced shapes.
//
// These must give bit-identical doubles to the reference's scalar CPU path,
// so each keeps the reference kernel's operation order and is compiled with
// -fmad=false (no contraction into FMA).  IEEE-rounded '/' and sqrt are the
// CUDA defaults (-prec-div / -prec-sqrt).
#pragma once

#include <cfloat>
#include <cstdint>

#include "geom_types.h"

// Two kernel sets are compiled from these sources: VGN_SECTIONS=1 (namespace `sections`)
// handles phi sections of tubes, cones and polycones and phi/theta sections of spheres;
// VGN_SECTIONS=0 (namespace `full_ranges`) compiles that code out, for geometries whose
// shapes all span the full angular ranges.  The host picks the set per geometry.
#ifndef VGN_SECTIONS
#define VGN_SECTIONS 1
#endif
#ifndef VGN_BOOLEANS
#define VGN_BOOLEANS 0  // the kernel set carries the boolean solids' code (built without the sections')
#endif
#if VGN_BOOLEANS
#define VGN_KSET booleans
#elif VGN_SECTIONS
#define VGN_KSET sections
#else
#define VGN_KSET full_ranges
#endif

namespace vgn {
namespace dev {
inline namespace VGN_KSET {

constexpr double kTolerance     = 1e-9;
constexpr double kHalfTolerance = 0.5 * kTolerance;
constexpr double kPushTolerance = 1e-6;  // Math.h:28
constexpr double kInfLength     = DBL_MAX;
constexpr double kEpsilon       = DBL_EPSILON;

enum : int { kInsideE = 1, kSurfaceE = 2, kOutsideE = 3 };

struct D3 {
  double x, y, z;
};

__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }

// Transform<kGeneric,kGeneric> (Transformation3D.h:663-673, 729-735, 746-770): a point and a
// direction into the frame of a placement (translation t, row-major rotation r)
__device__ __forceinline__ D3 xf_point(const double *t, const double *r, D3 p)
{
  const double t0 = p.x - t[0], t1 = p.y - t[1], t2 = p.z - t[2];
  double l0 = t0 * r[0], l1 = t0 * r[1], l2 = t0 * r[2];
  l0 += t1 * r[3];
  l1 += t1 * r[4];
  l2 += t1 * r[5];
  l0 += t2 * r[6];
  l1 += t2 * r[7];
  l2 += t2 * r[8];
  return d3(l0, l1, l2);
}

// TransformDirection<kGeneric>
__device__ __forceinline__ D3 xf_dir(const double *r, D3 d)
{
  double l0 = d.x * r[0], l1 = d.x * r[1], l2 = d.x * r[2];
  l0 += d.y * r[3];
  l1 += d.y * r[4];
  l2 += d.y * r[5];
  l0 += d.z * r[6];
  l1 += d.z * r[7];
  l2 += d.z * r[8];
  return d3(l0, l1, l2);
}
__device__ __forceinline__ double vmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double vmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double min3(double a, double b, double c) { return vmin(vmin(a, b), c); }
__device__ __forceinline__ double max3(double a, double b, double c) { return vmax(vmax(a, b), c); }
// Global.h:166-178
__device__ __forceinline__ double nonzero_abs(double x) { return fabs(x) + 1.0e-30; }
__device__ __forceinline__ double nonzero(double x) { return x + copysign(1.0e-30, x); }
__device__ __forceinline__ double sgn(double x) { return copysign(1.0, x); }

// ---------------------------------------------------------------- Box
// kernel/BoxImplementation.h:73-167; row = fDimensions
__device__ __forceinline__ bool box_contains(const double *h, D3 p)
{
  return max3(fabs(p.x) - h[0], fabs(p.y) - h[1], fabs(p.z) - h[2]) < 0.0;
}

__device__ __forceinline__ int box_inside(const double *h, D3 p)
{
  const double dist = max3(fabs(p.x) - h[0], fabs(p.y) - h[1], fabs(p.z) - h[2]);
  int r             = dist < 0.0 ? kInsideE : kOutsideE;
  if (fabs(dist) < kHalfTolerance) r = kSurfaceE;
  return r;
}

__device__ __forceinline__ double box_dist_in(const double *h, D3 p, D3 d)
{
  const double ix = 1.0 / nonzero(d.x), iy = 1.0 / nonzero(d.y), iz = 1.0 / nonzero(d.z);
  const double sx = sgn(d.x), sy = sgn(d.y), sz = sgn(d.z);
  const double inx = -sx * h[0] - p.x, iny = -sy * h[1] - p.y, inz = -sz * h[2] - p.z;
  const double ox = sx * h[0] - p.x, oy = sy * h[1] - p.y, oz = sz * h[2] - p.z;
  const double absOrthogOut = fabs(min3(sx * ox, sy * oy, sz * oz));
  const double distOut      = min3(ox * ix, oy * iy, oz * iz);
  double distance           = max3(inx * ix, iny * iy, inz * iz);
  if (distance >= distOut || distOut <= kHalfTolerance || absOrthogOut <= kHalfTolerance) distance = kInfLength;
  return distance;
}

__device__ __forceinline__ double box_dist_out(const double *h, D3 p, D3 d)
{
  const double ix = 1.0 / nonzero(d.x), iy = 1.0 / nonzero(d.y), iz = 1.0 / nonzero(d.z);
  const double sx = sgn(d.x), sy = sgn(d.y), sz = sgn(d.z);
  const double safetyIn = max3(fabs(p.x) - h[0], fabs(p.y) - h[1], fabs(p.z) - h[2]);
  double distance       = min3((sx * h[0] - p.x) * ix, (sy * h[1] - p.y) * iy, (sz * h[2] - p.z) * iz);
  if (safetyIn > kHalfTolerance) distance = -1.0;
  return distance;
}

__device__ __forceinline__ double box_safe_in(const double *h, D3 p)
{
  return max3(fabs(p.x) - h[0], fabs(p.y) - h[1], fabs(p.z) - h[2]);
}

__device__ __forceinline__ double box_safe_out(const double *h, D3 p)
{
  return min3(h[0] - fabs(p.x), h[1] - fabs(p.y), h[2] - fabs(p.z));
}

// ---------------------------------------------------------------- Wedge
// evolution::Wedge (Wedge_Evolution.h) over a row::Wedge* block of doubles
constexpr double kPiD = 3.14159265358979323846;

// Wedge::IsOnSurfaceGeneric (Wedge_Evolution.h:341-354)
__device__ __forceinline__ bool wedge_on_surface(double ax, double ay, double nx, double ny, D3 p)
{
  if (!(ax * p.x + ay * p.y >= 0.)) return false;
  return fabs(nx * p.x + ny * p.y) < kTolerance;
}

// Wedge::GenericKernelForContainsAndInside (Wedge_Evolution.h:306-339)
template <bool FOR_INSIDE>
__device__ __forceinline__ void wedge_ci(const double *w, D3 p, bool &cin, bool &cout)
{
  const double startCheck = (-p.x * w[row::WedgeA1y] + p.y * w[row::WedgeA1x]);
  const double endCheck   = (-w[row::WedgeA2x] * p.y + w[row::WedgeA2y] * p.x);
  cout                    = startCheck < 0.;
  if (w[row::WedgeDPhi] < kPiD)
    cout = cout || endCheck < 0.;
  else
    cout = cout && endCheck < 0.;
  if (FOR_INSIDE) {
    const bool onSurface =
        wedge_on_surface(w[row::WedgeA1x], w[row::WedgeA1y], w[row::WedgeN1x], w[row::WedgeN1y], p) ||
        wedge_on_surface(w[row::WedgeA2x], w[row::WedgeA2y], w[row::WedgeN2x], w[row::WedgeN2y], p);
    cout = cout && !onSurface;
    cin  = !onSurface && !cout;
  }
}

// Wedge::SafetyToIn (Wedge_Evolution.h:374-391)
__device__ __forceinline__ double wedge_safe_in(const double *w, D3 p)
{
  const double dist1 = p.x * w[row::WedgeN1x] + p.y * w[row::WedgeN1y];
  const double dist2 = p.x * w[row::WedgeN2x] + p.y * w[row::WedgeN2y];
  const double m1 = -1 * dist1, m2 = -1 * dist2;
  if (w[row::WedgeDPhi] < kPiD) return m1 > m2 ? m1 : m2;
  return m1 < m2 ? m1 : m2;
}

// Wedge::SafetyToOut (Wedge_Evolution.h:356-372)
__device__ __forceinline__ double wedge_safe_out(const double *w, D3 p)
{
  const double dist1 = p.x * w[row::WedgeN1x] + p.y * w[row::WedgeN1y];
  const double dist2 = p.x * w[row::WedgeN2x] + p.y * w[row::WedgeN2y];
  if (w[row::WedgeDPhi] < kPiD) return dist1 < dist2 ? dist1 : dist2;
  return dist1 > dist2 ? dist1 : dist2;
}

// ---------------------------------------------------------------- Tube
// kernel/TubeImplementation.h (UniversalTube: rmin and phi treatment decided at run
// time, TubeTypes.h:91-139); row layout vgn::row::Tube*, the phi wedge at TubeWedge
namespace tb = row;

__device__ __forceinline__ bool tube_has_phi(const double *t) { return VGN_SECTIONS && t[tb::TubeDphi] < 2. * kPiD; }

// TubeUtilities::PointInCyclicalSector<..., onSurfaceT = false> (TubeImplementation.h:58-101);
// "smaller than pi" is dphi <= M_PI, decided at run time
__device__ __forceinline__ bool tube_in_sector(const double *t, double x, double y, bool includeSurface)
{
  const double *w         = t + tb::TubeWedge;
  const double startCheck = (-x * w[row::WedgeA1y] + y * w[row::WedgeA1x]);
  const double endCheck   = (-w[row::WedgeA2x] * y + w[row::WedgeA2y] * x);
  const double tol        = includeSurface ? -kHalfTolerance : kHalfTolerance;
  if (t[tb::TubeDphi] <= kPiD) return (startCheck >= tol) && (endCheck >= tol);
  return (startCheck >= tol) || (endCheck >= tol);
}

// CircleTrajectoryIntersection (TubeImplementation.h:103-160)
__device__ __forceinline__ void tube_circle(const double *t, double b, double c, D3 pos, D3 dir, bool largest,
                                            bool insector, double &dist, bool &ok)
{
  double delta = b * b - c;
  ok           = delta > 0.;
  if (largest) ok |= delta == 0.;
  if (!ok) delta = 0.;
  delta = sqrt(delta);
  if (!largest) delta = -delta;
  dist = -b + delta;
  ok &= dist >= -2 * kTolerance;
  if (!ok) return;
  if (insector) {
    const double hitz = pos.z + dist * dir.z;
    ok &= (fabs(hitz) <= t[tb::TubeZ]);
    if (!ok) return;
    if (tube_has_phi(t)) ok &= tube_in_sector(t, pos.x + dist * dir.x, pos.y + dist * dir.y, true);
  }
}

// PhiPlaneTrajectoryIntersection (TubeImplementation.h:249-301)
__device__ __forceinline__ void tube_phi_plane(const double *t, double alongX, double alongY, double normalX,
                                               double normalY, D3 pos, D3 dir, bool posdir, bool insector,
                                               double &dist, bool &ok)
{
  const double dirDotNorm = dir.x * normalX + dir.y * normalY;
  ok                      = insector ? (dirDotNorm > 0.) : (dirDotNorm < 0.);
  const double dirDotXY   = (dir.y * alongX - dir.x * alongY);
  dist                    = (alongY * pos.x - alongX * pos.y) / nonzero(dirDotXY);
  ok &= (dist * fabs(dirDotNorm)) > -kHalfTolerance;
  if (insector) {
    const double hitx = pos.x + dist * dir.x;
    const double hity = pos.y + dist * dir.y;
    const double hitz = pos.z + dist * dir.z;
    const double r2   = hitx * hitx + hity * hity;
    ok &= fabs(hitz) <= t[tb::TubeTolOz] && (r2 >= t[tb::TubeTolOrmin2]) && (r2 <= t[tb::TubeTolOrmax2]);
    if (posdir) ok = ok && (hitx * alongX + hity * alongY) > 0.;
  } else if (posdir) {
    const double hitx = pos.x + dist * dir.x;
    const double hity = pos.y + dist * dir.y;
    ok                = ok && (hitx * alongX + hity * alongY) >= 0.;
  }
}

// The two phi-plane candidates that end DistanceToIn (`in`, TubeImplementation.h:656-679) and
// DistanceToOut (790-821) of a tube section.  The sector type of UniversalTube is unknown at
// compile time, so both planes are checked, with the positive-direction test.  In both kernels
// the first plane's candidate is taken when it is below the distance so far, then the second's
// when it is below that; out of line, since only phi sections take it.
__device__ __noinline__ double tube_phi_planes(const double *t, D3 p, D3 d, double distance, bool in)
{
  const double *w = t + tb::TubeWedge;
  double dist_phi;
  bool ok_phi;
  tube_phi_plane(t, w[row::WedgeA1x], w[row::WedgeA1y], w[row::WedgeN1x], w[row::WedgeN1y], p, d, true, in,
                 dist_phi, ok_phi);
  if (ok_phi && dist_phi < distance) distance = dist_phi;
  tube_phi_plane(t, w[row::WedgeA2x], w[row::WedgeA2y], w[row::WedgeN2x], w[row::WedgeN2y], p, d, true, in,
                 dist_phi, ok_phi);
  if (ok_phi && dist_phi < distance) distance = dist_phi;
  return distance;
}

// PhiPlaneSafety<inside = false> (TubeImplementation.h:210-247), UniversalTube
__device__ __forceinline__ double tube_phi_safety(const double *t, D3 pos)
{
  const double *w = t + tb::TubeWedge;
  double safety   = t[tb::TubeDphi] > kPiD ? sqrt(pos.x * pos.x + pos.y * pos.y) : kInfLength;
  const double phi1 = pos.x * w[row::WedgeA1y] - pos.y * w[row::WedgeA1x];  // PerpDist2D
  if (phi1 > -kHalfTolerance && phi1 < safety) safety = phi1;
  double phi2 = pos.x * w[row::WedgeA2y] - pos.y * w[row::WedgeA2x];
  phi2 *= -1;
  if (phi2 > -kHalfTolerance && phi2 < safety) safety = phi2;
  return safety;
}

// DistanceToInKernel (TubeImplementation.h:504-681)
__device__ __forceinline__ double tube_dist_in_kernel(const double *t, D3 p, D3 d)
{
  const bool hasrmin = t[tb::TubeRmin] > 0;
  const bool hasphi  = tube_has_phi(t);
  bool done          = false;
  double distance    = kInfLength;
  double distz       = fabs(p.z) - t[tb::TubeZ];
  done |= distz > kHalfTolerance && p.z * d.z >= 0;
  const double rsq   = p.x * p.x + p.y * p.y;
  const double rdotn = p.x * d.x + p.y * d.y;
  done |= rsq > t[tb::TubeTolIrmax2] && rdotn >= 0;
  if (done) return distance;

  distance    = -1.0;
  bool inside = distz < -kHalfTolerance;
  inside &= rsq < t[tb::TubeTolIrmax2];
  if (hasrmin) inside &= rsq > t[tb::TubeTolIrmin2];
  if (hasphi && inside) inside &= tube_in_sector(t, p.x, p.y, false);
  done |= inside;
  if (done) return distance;

  distance = kInfLength;
  distz /= nonzero_abs(d.z);
  const double hitx = p.x + distz * d.x;
  const double hity = p.y + distz * d.y;
  const double r2   = hitx * hitx + hity * hity;
  bool okz          = distz > -kHalfTolerance && (p.z * d.z < 0);
  okz &= (r2 <= t[tb::TubeRmax2]);
  if (hasrmin) okz &= (t[tb::TubeRmin2] <= r2);
  if (hasphi && okz) okz &= tube_in_sector(t, hitx, hity, true);
  if (!done && okz) distance = distz;
  done |= okz;

  const double rho = p.x * p.x + p.y * p.y;
  bool onsurf = (rho >= t[tb::TubeTolIrmax2]) && (rho <= t[tb::TubeTolOrmax2]) &&
                (fabs(p.z) < (t[tb::TubeZ] + kTolerance)) && (d.x * p.x + d.y * p.y + d.z * 0. <= 0.);
  if (hasrmin)
    onsurf |= (rho >= t[tb::TubeTolOrmin2]) && (rho <= t[tb::TubeTolIrmin2]) &&
              (fabs(p.z) < (t[tb::TubeZ] + kTolerance)) && (d.x * -p.x + d.y * -p.y + d.z * 0. <= 0.);
  if (hasphi) onsurf = onsurf && tube_in_sector(t, p.x, p.y, true);
  if (!done && onsurf) distance = 0.;
  done |= onsurf;
  if (done) return distance;

  const double invnsq = 1. / nonzero(1. - d.z * d.z);
  const double b      = invnsq * rdotn;
  const double crmax  = invnsq * (rsq - t[tb::TubeRmax2]);
  double dist_rmax;
  bool ok_rmax;
  tube_circle(t, b, crmax, p, d, false, true, dist_rmax, ok_rmax);
  ok_rmax &= dist_rmax < distance;
  if (!done && ok_rmax) distance = dist_rmax;
  done |= ok_rmax;
  if (done) return distance;
  if (hasrmin) {
    const double crmin = invnsq * (rsq - t[tb::TubeRmin2]);
    double dist_rmin;
    bool ok_rmin;
    tube_circle(t, b, crmin, p, d, true, true, dist_rmin, ok_rmin);
    ok_rmin &= dist_rmin < distance;
    if (!done && ok_rmin) distance = dist_rmin;
  }
  if (hasphi) distance = tube_phi_planes(t, p, d, distance, true);
  return distance;
}

// DistanceToIn with the far-point pre-move (TubeImplementation.h:475-502)
__device__ __forceinline__ double tube_dist_in(const double *t, D3 pt, D3 d)
{
  D3 p                = pt;
  const double ptDist = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double distToMove   = 0.;
  const double order  = 100.;
  if (ptDist > order * t[tb::TubeMaxVal]) {
    distToMove = ptDist - order * t[tb::TubeMaxVal];
    p          = d3(p.x + distToMove * d.x, p.y + distToMove * d.y, p.z + distToMove * d.z);
  }
  double distance = tube_dist_in_kernel(t, p, d);
  distance += distToMove;
  return distance;
}

// DistanceToOut (TubeImplementation.h:683-823)
__device__ __forceinline__ double tube_dist_out(const double *t, D3 p, D3 d)
{
  const bool hasrmin = t[tb::TubeRmin] > 0;
  const bool hasphi  = tube_has_phi(t);
  const double fz    = t[tb::TubeZ];
  double distz       = fz - fabs(p.z);
  if (distz < -kHalfTolerance) return -1.;
  const double rsq   = p.x * p.x + p.y * p.y;
  const double rdotn = d.x * p.x + d.y * p.y;
  double crmax       = rsq - t[tb::TubeRmax2];
  double crmin       = rsq;
  if (crmax > 2.0 * kTolerance * t[tb::TubeRmax]) return -1.;
  if (hasrmin) {
    crmin -= t[tb::TubeRmin2];
    if (crmin < -2.0 * kTolerance * t[tb::TubeRmin]) return -1.;
  }
  if (hasphi) {
    bool cin = false, cout = false;
    wedge_ci<true>(t + tb::TubeWedge, p, cin, cout);
    if (cout) return -1.;
  }
  double distance      = kInfLength;
  const double invdirz = 1. / nonzero(d.z);
  distz                = (fz - p.z) * invdirz;
  if (d.z < 0) distz = (-fz - p.z) * invdirz;
  if (d.z != 0. && distz < distance) distance = distz;
  const double invnsq = 1. / nonzero(1. - d.z * d.z);
  const double b      = invnsq * rdotn;
  if (hasrmin) {
    double dist_rmin;
    bool ok_rmin;
    crmin *= invnsq;
    tube_circle(t, b, crmin, p, d, false, false, dist_rmin, ok_rmin);
    if (ok_rmin && dist_rmin < distance) distance = dist_rmin;
  }
  double dist_rmax;
  bool ok_rmax;
  crmax *= invnsq;
  tube_circle(t, b, crmax, p, d, true, false, dist_rmax, ok_rmax);
  if (ok_rmax && dist_rmax < distance) distance = dist_rmax;
  if (hasphi) distance = tube_phi_planes(t, p, d, distance, false);
  return distance;
}

// SafetyToInOld (TubeImplementation.h:912-938; TUBE_SAFETY_OLD is defined at line 14)
__device__ __forceinline__ double tube_safe_in(const double *t, D3 p)
{
  double safety         = fabs(p.z) - t[tb::TubeZ];
  const double r        = sqrt(p.x * p.x + p.y * p.y);
  const double safermax = r - t[tb::TubeRmax];
  if (safermax > safety) safety = safermax;
  if (t[tb::TubeRmin] > 0) {
    const double safermin = t[tb::TubeRmin] - r;
    if (safermin > safety) safety = safermin;
  }
  if (tube_has_phi(t)) {
    const bool insector = tube_in_sector(t, p.x, p.y, false);
    if (insector) return safety;
    const double safephi = tube_phi_safety(t, p);
    if (!insector && safephi < kInfLength && safephi > safety) safety = safephi;
  }
  return safety;
}

// SafetyToOutOld (TubeImplementation.h:940-966)
__device__ __forceinline__ double tube_safe_out(const double *t, D3 p)
{
  double safety         = t[tb::TubeZ] - fabs(p.z);
  const double r        = sqrt(p.x * p.x + p.y * p.y);
  const double safermax = t[tb::TubeRmax] - r;
  if (safermax < safety) safety = safermax;
  if (t[tb::TubeRmin] > 0) {
    const double safermin = r - t[tb::TubeRmin];
    if (safermin < safety) safety = safermin;
  }
  if (tube_has_phi(t)) {
    const double safephi = wedge_safe_out(t + tb::TubeWedge, p);
    if (safephi < safety) safety = safephi;
  }
  return safety;
}

// GenericKernelForContainsAndInside (TubeImplementation.h:392-450)
__device__ __forceinline__ void tube_generic_ci(const double *t, D3 p, bool forinside, bool &cin, bool &cout)
{
  const double fz = t[tb::TubeZ], rmax = t[tb::TubeRmax], rmin = t[tb::TubeRmin];
  const double absz = fabs(p.z);
  cout = absz > (forinside ? fz + kHalfTolerance : fz);
  if (forinside) cin = absz < fz - kHalfTolerance;
  if (cout) return;
  const double r2 = p.x * p.x + p.y * p.y;
  cout |= r2 > (forinside ? rmax * (rmax + 2.0 * kTolerance) : rmax * rmax);
  if (forinside) cin &= r2 < fabs(rmax * (rmax - 2.0 * kTolerance));
  if (cout) return;
  if (rmin > 0) {
    cout |= r2 <= (forinside ? fabs(rmin * (rmin - 2.0 * kTolerance)) : rmin * rmin);
    if (forinside) cin &= r2 > rmin * (rmin + 2.0 * kTolerance);
    if (cout) return;
  }
  if (tube_has_phi(t)) {
    bool cinphi = false, coutphi = false;
    if (forinside)
      wedge_ci<true>(t + tb::TubeWedge, p, cinphi, coutphi);
    else
      wedge_ci<false>(t + tb::TubeWedge, p, cinphi, coutphi);
    cout |= coutphi;
    if (forinside) cin &= cinphi;
  }
}

__device__ __forceinline__ bool tube_contains(const double *t, D3 p)
{
  bool cin = false, cout = false;
  tube_generic_ci(t, p, false, cin, cout);
  return !cout;
}

__device__ __forceinline__ int tube_inside(const double *t, D3 p)
{
  bool cin = false, cout = false;
  tube_generic_ci(t, p, true, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// ---------------------------------------------------------------- Cone
// kernel/ConeImplementation.h:117-516, ConeUtilities.h:64-813 (the scalar ConeHelpers<double>
// specialisation); UniversalCone: rmin and phi treatment at run time; row layout vgn::row::Cone*
constexpr double kConeTolerance = 1e-7;

// MakePlus/MinusTolerantSquare<true> (kernel/GenericKernels.h:65-82)
__device__ __forceinline__ double plus_tol_sq(double x, double tol) { return x * (x + 2.0 * tol); }
__device__ __forceinline__ double minus_tol_sq(double x, double tol) { return fabs(x * (x - 2.0 * tol)); }

__device__ __forceinline__ bool cone_has_rmin(const double *c) { return c[row::ConeRmin1] > 0 || c[row::ConeRmin2] > 0; }

// GetRadiusOfConeAtPoint (ConeUtilities.h:116-137)
__device__ __forceinline__ double cone_radius(const double *c, double z, bool inner)
{
  if (inner)
    return c[row::ConeRmin1] == c[row::ConeRmin2] ? c[row::ConeRmin1]
                                                    : c[row::ConeInnerSlope] * z + c[row::ConeInnerOffset];
  return c[row::ConeOrigRmax1] == c[row::ConeOrigRmax2] ? c[row::ConeOrigRmax1]
                                                          : c[row::ConeOuterSlope] * z + c[row::ConeOuterOffset];
}

__device__ __forceinline__ bool cone_has_phi(const double *c) { return VGN_SECTIONS && c[row::ConeDPhi] < 2. * kPiD; }

// PointInCyclicalSector<..., onSurfaceT = false> (ConeUtilities.h:64-114); "smaller than pi"
// is dphi <= M_PI, decided at run time
__device__ __forceinline__ bool cone_in_sector(const double *c, double x, double y, bool includeSurface)
{
  const double startCheck = (-x * c[row::ConeAP1y]) + (y * c[row::ConeAP1x]);
  const double endCheck   = (-c[row::ConeAP2x] * y) + (c[row::ConeAP2y] * x);
  const double tol        = includeSurface ? -kConeTolerance : kConeTolerance;
  if (c[row::ConeDPhi] <= kPiD) return (startCheck >= tol) && (endCheck >= tol);
  return (startCheck >= tol) || (endCheck >= tol);
}

// PhiPlaneTrajectoryIntersection (ConeUtilities.h:155-204)
__device__ __forceinline__ void cone_phi_plane(const double *c, double alongX, double alongY, double normalX,
                                               double normalY, D3 pos, D3 dir, bool posdir, bool insector,
                                               double &dist, bool &ok)
{
  dist = kInfLength;
  if (insector)
    ok = ((dir.x * normalX) + (dir.y * normalY) > 0.);
  else
    ok = ((dir.x * normalX) + (dir.y * normalY) < 0.);
  const double dirDotXY = (dir.y * alongX) - (dir.x * alongY);
  if (dirDotXY != 0) dist = ((alongY * pos.x) - (alongX * pos.y)) / nonzero(dirDotXY);
  ok &= dist > -kConeTolerance;
  if (insector) {
    const double hitx          = pos.x + dist * dir.x;
    const double hity          = pos.y + dist * dir.y;
    const double hitz          = pos.z + dist * dir.z;
    const double r2            = (hitx * hitx) + (hity * hity);
    const double innerRadIrTol = cone_radius(c, hitz, true) + kTolerance;
    const double outerRadIrTol = cone_radius(c, hitz, false) - kTolerance;
    ok &= fabs(hitz) <= c[row::ConeTolIz] && (r2 >= innerRadIrTol * innerRadIrTol) &&
          (r2 <= outerRadIrTol * outerRadIrTol);
    if (posdir) ok = ok && ((hitx * alongX) + (hity * alongY)) > 0.;
  } else if (posdir) {
    const double hitx = pos.x + dist * dir.x;
    const double hity = pos.y + dist * dir.y;
    ok                = ok && ((hitx * alongX) + (hity * alongY)) >= 0.;
  }
}

// The two phi-plane candidates that end DistanceToIn (`in`, ConeImplementation.h:233-254) and
// DistanceToOut (336-364) of a cone section: the sector type of UniversalCone is unknown at
// compile time, so both planes are checked, with the positive-direction test; the first
// plane's candidate is taken when below the distance so far, then the second's when below
// that.  Out of line, since only phi sections take it.
__device__ __noinline__ double cone_phi_planes(const double *c, D3 p, D3 d, double distance, bool in)
{
  const double *w = c + row::ConeWedge;
  double dist_phi;
  bool ok_phi;
  cone_phi_plane(c, c[row::ConeAP1x], c[row::ConeAP1y], w[row::WedgeN1x], w[row::WedgeN1y], p, d, true, in,
                 dist_phi, ok_phi);
  if (ok_phi && dist_phi < distance) distance = dist_phi;
  cone_phi_plane(c, c[row::ConeAP2x], c[row::ConeAP2y], w[row::WedgeN2x], w[row::WedgeN2y], p, d, true, in,
                 dist_phi, ok_phi);
  if (ok_phi && dist_phi < distance) distance = dist_phi;
  return distance;
}

// GetNormal (ConeUtilities.h:206-238)
__device__ __forceinline__ D3 cone_normal(const double *c, D3 p, bool inner)
{
  const double rho = sqrt(p.x * p.x + p.y * p.y);
  if (inner) {
    if ((c[row::ConeRmin1] == c[row::ConeRmin2]) && (c[row::ConeRmin1] != 0.)) return d3(-p.x, -p.y, 0.);
    return d3(-p.x, -p.y, c[row::ConeZNormInner] * (rho * c[row::ConeSecRMin]));
  }
  if ((c[row::ConeRmax1] == c[row::ConeRmax2]) && (c[row::ConeRmax1] != 0.)) return d3(p.x, p.y, 0.);
  return d3(p.x, p.y, c[row::ConeZNormOuter] * (rho * c[row::ConeSecRMax]));
}

__device__ __forceinline__ double dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// IsOnConicalSurface (ConeUtilities.h:240-255)
__device__ __forceinline__ bool cone_on_surface(const double *c, D3 p, bool inner)
{
  const double rho      = p.x * p.x + p.y * p.y;
  const double coneRad  = cone_radius(c, p.z, inner);
  const double coneRad2 = coneRad * coneRad;
  const double tol      = inner ? c[row::ConeInnerTol] : c[row::ConeOuterTol];
  return (rho >= (coneRad2 - tol * coneRad)) && (rho <= (coneRad2 + tol * coneRad)) &&
         (fabs(p.z) < (c[row::ConeDz] + kConeTolerance));
}

// ConeHelpers<double>::DetectIntersectionAndCalculateDistanceToConicalSurface (ConeUtilities.h:591-762)
template <bool PHI = true>
__device__ __forceinline__ bool cone_conical(const double *c, D3 p, D3 d, bool fordistin, bool inner, double &distance)
{
  distance          = kInfLength;
  const bool onsurf = cone_on_surface(c, p, inner);
  const D3 n        = cone_normal(c, p, inner);
  const double dn   = dot3(d, n);
  if (onsurf && fabs(dn) == 0.) return false;
  if (onsurf) {
    bool moving = fordistin ? (dn <= 0.) : (dn >= 0.);
    if ((PHI && cone_has_phi(c))) moving = cone_in_sector(c, p.x, p.y, true) && moving;
    if (moving) {
      distance = 0.;
      return true;
    }
  }
  const double pDotV2D = p.x * d.x + p.y * d.y;
  const double dz      = c[row::ConeDz];
  double a, b, cc;
  bool ok = false;
  if (inner) {
    if (c[row::ConeRmin1] == c[row::ConeRmin2]) {
      b  = pDotV2D;
      a  = d.x * d.x + d.y * d.y;
      cc = (p.x * p.x + p.y * p.y) - c[row::ConeRmin2] * c[row::ConeRmin2];
    } else {
      const double tanA  = c[row::ConeTanInnerApex];
      const double newPz = (c[row::ConeRmin2] > c[row::ConeRmin1]) ? (p.z + dz + c[row::ConeInnerApex]) * tanA
                                                                     : (p.z - dz - c[row::ConeInnerApex]) * tanA;
      const double dirT  = d.z * tanA;
      a  = (d.x * d.x) + (d.y * d.y) - dirT * dirT;
      b  = pDotV2D - (newPz * dirT);
      cc = (p.x * p.x + p.y * p.y) - (newPz * newPz);
    }
    const double b2 = b * b, ac = a * cc;
    if (b2 < ac) return false;
    const double delta = sqrt(b2 - ac);
    if (fordistin) {
      distance = (b >= 0.) ? (cc / nonzero(-b - delta)) : (-b + delta) / nonzero(a);
    } else {
      if (b == 0. && delta == 0.) return false;
      distance = (b >= 0.) ? (-b - delta) / nonzero(a) : (cc / nonzero(-b + delta));
    }
    if (distance < 0.) return false;
    const double newZ = p.z + (d.z * distance);
    ok                = (fabs(newZ) < dz);
  } else {
    if (c[row::ConeOrigRmax1] == c[row::ConeOrigRmax2]) {
      a  = d.x * d.x + d.y * d.y;
      b  = pDotV2D;
      cc = ((p.x * p.x + p.y * p.y) - c[row::ConeOrigRmax2] * c[row::ConeOrigRmax2]);
    } else {
      const double tanA  = c[row::ConeTanOuterApex];
      const double newPz = (c[row::ConeOrigRmax2] > c[row::ConeOrigRmax1])
                               ? (p.z + dz + c[row::ConeOuterApex]) * tanA
                               : (p.z - dz - c[row::ConeOuterApex]) * tanA;
      const double dirT  = d.z * tanA;
      a  = d.x * d.x + d.y * d.y - dirT * dirT;
      b  = (pDotV2D - (newPz * dirT));
      cc = ((p.x * p.x + p.y * p.y) - (newPz * newPz));
    }
    const double b2 = b * b, ac = a * cc, d2 = b2 - ac;
    if (d2 < 0) return false;
    const double delta = sqrt(d2);
    if (fordistin) {
      if (b == 0. && delta == 0.) return false;
      distance = (b > 0.) ? (-b - delta) / nonzero(a) : (cc / nonzero(-b + delta));
      const double newZ = p.z + (d.z * distance);
      ok                = (fabs(newZ) < dz + kHalfTolerance);
    } else {
      distance = (b < 0.) ? (-b + delta) / nonzero(a) : (cc / nonzero(-b - delta));
      ok       = distance > 0.;
    }
    if (distance < 0.) return false;
  }
  if ((PHI && cone_has_phi(c))) {
    double hitx = 0, hity = 0;
    if (distance < kInfLength) {
      hitx = p.x + distance * d.x;
      hity = p.y + distance * d.y;
    }
    ok &= (cone_in_sector(c, hitx, hity, true) && (distance < kInfLength));
  }
  return ok;
}

// DistanceToIn (ConeImplementation.h:117-255)
template <bool PHI = true>
__device__ __forceinline__ double cone_dist_in(const double *c, D3 p, D3 d)
{
  const bool hasrmin = cone_has_rmin(c);
  const bool hasphi  = (PHI && cone_has_phi(c));
  const double dz    = c[row::ConeDz];
  double distance    = kInfLength;
  double distz       = fabs(p.z) - dz;
  if ((distz > kConeTolerance && (p.z * d.z) >= 0.) || (fabs(distz) < kConeTolerance && (p.z * d.z) > 0.))
    return distance;
  const double outerRad = cone_radius(c, p.z, false);
  const double rsq      = p.x * p.x + p.y * p.y;
  if ((rsq > minus_tol_sq(outerRad, c[row::ConeOuterTol])) && (dot3(d, cone_normal(c, p, false)) >= 0.))
    return distance;
  bool inside = distz < -kConeTolerance;
  inside &= rsq < minus_tol_sq(outerRad, c[row::ConeOuterTol]);
  if (hasrmin) inside &= rsq > plus_tol_sq(cone_radius(c, p.z, true), c[row::ConeInnerTol]);
  if (hasphi) inside &= cone_in_sector(c, p.x, p.y, false);
  if (inside) return -1.0;
  distance = kInfLength;
  distz /= nonzero(fabs(d.z));
  const double hitx = p.x + distz * d.x;
  const double hity = p.y + distz * d.y;
  const double r2   = (hitx * hitx) + (hity * hity);
  bool top = (p.z >= c[row::ConeTolIz]) && (r2 <= c[row::ConeSqRmax2] + kTolerance);
  bool bot = (p.z <= -c[row::ConeTolIz]) && (r2 <= c[row::ConeSqRmax1] + kTolerance);
  bool okz = top || bot;
  if (hasrmin) {
    top &= (r2 >= c[row::ConeSqRmin2] - kTolerance);
    bot &= (r2 >= c[row::ConeSqRmin1] - kTolerance);
    okz &= (top || bot);
  }
  if (hasphi) okz &= cone_in_sector(c, hitx, hity, true);
  if (okz) return distz;
  double dr;
  bool ok = cone_conical<PHI>(c, p, d, true, false, dr);
  ok &= dr < distance;
  if (ok) return dr;
  if (hasrmin) {
    ok = cone_conical<PHI>(c, p, d, true, true, dr);
    ok &= dr < distance;
    if (ok) distance = dr;
  }
  if (hasphi) distance = cone_phi_planes(c, p, d, distance, true);
  return distance;
}

// DistanceToOut (ConeImplementation.h:257-366)
template <bool PHI = true>
__device__ __forceinline__ double cone_dist_out(const double *c, D3 p, D3 d)
{
  const bool hasrmin = cone_has_rmin(c);
  const double dz    = c[row::ConeDz];
  const double distz = fabs(p.z) - dz;
  bool outside       = distz > kConeTolerance;
  const double rsq   = p.x * p.x + p.y * p.y;
  outside |= rsq > plus_tol_sq(cone_radius(c, p.z, false), c[row::ConeOuterTol]);
  if (outside) return -1.0;
  if (hasrmin) {
    outside |= rsq < minus_tol_sq(cone_radius(c, p.z, true), c[row::ConeInnerTol]);
    if (outside) return -1.0;
  }
  const bool up = d.z > 0., down = d.z < 0.;
  if ((up && p.z > 0. && fabs(distz) < kConeTolerance) || (down && p.z < 0. && fabs(distz) < kConeTolerance))
    return distz;
  double distance      = kInfLength;
  const double dirZInv = 1. / nonzero(d.z);
  if (up) distance = (dz - p.z) * dirZInv;
  if (down) distance = (-dz - p.z) * dirZInv;
  double dr;
  bool ok = cone_conical<PHI>(c, p, d, false, false, dr);
  if (ok && dr < distance) distance = dr;
  if (hasrmin) {
    ok = cone_conical<PHI>(c, p, d, false, true, dr);
    if (ok && dr < distance) distance = dr;
  }
  if ((PHI && cone_has_phi(c))) {
    // the outside test's phi part (ConeImplementation.h:293-297) only runs where the point is
    // already outside, so it never changes the result of the scalar kernel
    const double *w    = c + row::ConeWedge;
    const bool onStart = wedge_on_surface(w[row::WedgeA1x], w[row::WedgeA1y], w[row::WedgeN1x], w[row::WedgeN1y], p);
    const bool onEnd   = wedge_on_surface(w[row::WedgeA2x], w[row::WedgeA2y], w[row::WedgeN2x], w[row::WedgeN2y], p);
    if ((onStart && (d.x * -w[row::WedgeN1x] + d.y * -w[row::WedgeN1y] + d.z * -0.) > 0.) ||
        (onEnd && (d.x * -w[row::WedgeN2x] + d.y * -w[row::WedgeN2y] + d.z * -0.) > 0.))
      return 0.;
    distance = cone_phi_planes(c, p, d, distance, false);
  }
  if (distance < 0. && fabs(distance) < kTolerance) distance = 0.;
  return distance;
}

// SafeDistanceToConicalSurface (ConeImplementation.h:502-516)
__device__ __forceinline__ double cone_safe_surface(const double *c, D3 p, bool inner)
{
  const double rho = sqrt(p.x * p.x + p.y * p.y);
  if (inner) {
    const double pRMin = c[row::ConeTanRMin] * p.z + (c[row::ConeRmin1] + c[row::ConeRmin2]) * 0.5;
    return (rho - pRMin) * c[row::ConeInvSecRMin];
  }
  const double pRMax = c[row::ConeTanRMax] * p.z + (c[row::ConeRmax1] + c[row::ConeRmax2]) * 0.5;
  return (pRMax - rho) * c[row::ConeInvSecRMax];
}

// SafetyToIn (ConeImplementation.h:368-432)
template <bool PHI = true>
__device__ __forceinline__ double cone_safe_in(const double *c, D3 p)
{
  const bool hasrmin = cone_has_rmin(c);
  const double distz = fabs(p.z) - c[row::ConeDz];
  const double rsq   = p.x * p.x + p.y * p.y;
  bool inside        = distz < -kConeTolerance;
  inside &= rsq < minus_tol_sq(cone_radius(c, p.z, false), c[row::ConeOuterTol]);
  if (hasrmin) inside &= rsq > plus_tol_sq(cone_radius(c, p.z, true), c[row::ConeInnerTol]);
  if ((PHI && cone_has_phi(c)) && inside) inside &= cone_in_sector(c, p.x, p.y, false);
  if (inside) return -1.0;
  const double safeZ = fabs(p.z) - c[row::ConeDz];
  const double so    = -cone_safe_surface(c, p, false);
  const double si    = hasrmin ? -cone_safe_surface(c, p, true) : -kInfLength;
  double safety      = vmax(safeZ, vmax(so, si));
  if ((PHI && cone_has_phi(c))) safety = vmax(wedge_safe_in(c + row::ConeWedge, p), safety);
  if (fabs(safety) < kTolerance) safety = 0.;
  return safety;
}

// SafetyToOut (ConeImplementation.h:434-499)
template <bool PHI = true>
__device__ __forceinline__ double cone_safe_out(const double *c, D3 p)
{
  const bool hasrmin = cone_has_rmin(c);
  const double distz = fabs(p.z) - c[row::ConeDz];
  const double rsq   = p.x * p.x + p.y * p.y;
  bool outside       = distz > kConeTolerance;
  outside |= rsq > plus_tol_sq(cone_radius(c, p.z, false), c[row::ConeOuterTol]);
  if (hasrmin) outside |= rsq < minus_tol_sq(cone_radius(c, p.z, true), c[row::ConeInnerTol]);
  if (outside) return -1.0;
  const double safeZ = c[row::ConeDz] - fabs(p.z);
  const double so    = cone_safe_surface(c, p, false);
  const double si    = hasrmin ? cone_safe_surface(c, p, true) : kInfLength;
  double safety      = vmin(safeZ, vmin(so, si));
  if ((PHI && cone_has_phi(c))) safety = vmin(wedge_safe_out(c + row::ConeWedge, p), safety);
  if (fabs(safety) < kTolerance) safety = 0.;
  return safety;
}

// ConeHelpers<double>::GenericKernelForContainsAndInside (ConeUtilities.h:764-813)
template <bool PHI = true>
__device__ __forceinline__ void cone_generic_ci(const double *c, D3 p, bool forinside, bool &cin, bool &cout)
{
  const double dz = c[row::ConeDz], absz = fabs(p.z);
  cout = absz > (forinside ? dz + kConeTolerance : dz);
  if (forinside) cin = absz < dz - kConeTolerance;
  if (cout) return;
  const double r2   = p.x * p.x + p.y * p.y;
  const double rmax = (c[row::ConeOrigRmax1] == c[row::ConeOrigRmax2])
                          ? c[row::ConeOrigRmax1]
                          : c[row::ConeOuterSlope] * p.z + c[row::ConeOuterOffset];
  cout |= r2 > (forinside ? plus_tol_sq(rmax, c[row::ConeOuterTol]) : rmax * rmax);
  if (forinside) cin &= r2 < minus_tol_sq(rmax, c[row::ConeOuterTol]);
  if (cout) return;
  if (cone_has_rmin(c)) {
    const double rmin = c[row::ConeInnerSlope] * p.z + c[row::ConeInnerOffset];
    cout |= r2 <= (forinside ? minus_tol_sq(rmin, c[row::ConeInnerTol]) : rmin * rmin);
    if (forinside) cin &= r2 > plus_tol_sq(rmin, c[row::ConeInnerTol]);
    if (cout) return;
  }
  if ((PHI && cone_has_phi(c))) {
    bool cinphi = false, coutphi = false;
    if (forinside)
      wedge_ci<true>(c + row::ConeWedge, p, cinphi, coutphi);
    else
      wedge_ci<false>(c + row::ConeWedge, p, cinphi, coutphi);
    cout |= coutphi;
    if (forinside) cin &= cinphi;
  }
}

template <bool PHI = true>
__device__ __forceinline__ bool cone_contains(const double *c, D3 p)
{
  bool cin = false, cout = false;
  cone_generic_ci<PHI>(c, p, false, cin, cout);
  return !cout;
}

template <bool PHI = true>
__device__ __forceinline__ int cone_inside(const double *c, D3 p)
{
  bool cin = false, cout = false;
  cone_generic_ci<PHI>(c, p, true, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// ---------------------------------------------------------------- Trd
// UniversalTrd (volumes/kernel/TrdImplementation.h); the default build sets
// VECGEOM_NO_SPECIALIZATION, so every Trd takes the runtime dy1 != dy2 test.
namespace td = row;
constexpr double kTiny = 1e-30;  // base/Math.h:51

__device__ __forceinline__ bool trd_varying_y(const double *t) { return t[td::TrdDy1] != t[td::TrdDy2]; }

// TrdUtilities::FaceTrajectoryIntersection (TrdImplementation.h:80-138); dist is
// written only once the direction faces the plane.
template <bool FOR_Y, bool MIRRORED, bool TO_INSIDE>
__device__ __forceinline__ bool trd_face(const double *t, D3 pos, D3 dir, double &dist)
{
  double alongV, posV, dirV, posK, dirK, fV, fK, halfKplus, v1;
  if (FOR_Y) {
    alongV = t[td::TrdY2minusY1]; v1 = t[td::TrdDy1]; posV = pos.y; posK = pos.x; dirV = dir.y; dirK = dir.x;
    fK = t[td::TrdFx]; fV = t[td::TrdFy]; halfKplus = t[td::TrdHalfX1plusX2];
  } else {
    alongV = t[td::TrdX2minusX1]; v1 = t[td::TrdDx1]; posV = pos.x; posK = pos.y; dirV = dir.x; dirK = dir.y;
    fK = t[td::TrdFy]; fV = t[td::TrdFx]; halfKplus = t[td::TrdHalfY1plusY2];
  }
  if (MIRRORED) {
    posV *= -1.;
    dirV *= -1.;
  }
  const double ndotv = dirV + fV * dir.z;
  bool ok            = TO_INSIDE ? ndotv < 0. : ndotv > 0.;
  if (!ok) return false;
  const double fdz    = t[td::TrdDz];
  const double alongZ = 2.0 * fdz;
  dist = (alongZ * (posV - v1) - alongV * (pos.z + fdz)) / (dir.z * alongV - dirV * alongZ + kTiny);
  ok   = dist > (0. - kHalfTolerance);
  if (ok) {
    const double hitz = pos.z + dist * dir.z;
    ok                = fabs(hitz) <= fdz;
    const double hitk = posK + dist * dirK;
    const double dK   = halfKplus - fK * hitz;
    ok                = ok && fabs(hitk) <= dK;
    if (ok && fabs(dist) < kHalfTolerance) dist = 0.0;
  }
  return ok;
}

// TrdUtilities::Safety (TrdImplementation.h:140-168)
__device__ __forceinline__ double trd_safety(const double *t, D3 p, bool inside)
{
  double dist        = t[td::TrdDz] - fabs(p.z);
  const double distx = t[td::TrdHalfX1plusX2] - t[td::TrdFx] * p.z;
  const double safx  = (distx - fabs(p.x)) * t[td::TrdCalfX];
  if (distx >= 0 && safx < dist) dist = safx;
  if (trd_varying_y(t)) {
    const double disty = t[td::TrdHalfY1plusY2] - t[td::TrdFy] * p.z;
    const double safy  = (disty - fabs(p.y)) * t[td::TrdCalfY];
    if (disty >= 0 && safy < dist) dist = safy;
  } else {
    const double safy = t[td::TrdDy1] - fabs(p.y);
    if (safy < dist) dist = safy;
  }
  return inside ? dist : -dist;
}
__device__ __forceinline__ double trd_safe_in(const double *t, D3 p) { return trd_safety(t, p, false); }
__device__ __forceinline__ double trd_safe_out(const double *t, D3 p) { return trd_safety(t, p, true); }

// TrdUtilities::UnplacedInside (TrdImplementation.h:170-214), general y test
template <bool SURFACE>
__device__ __forceinline__ void trd_unplaced_inside(const double *t, D3 p, bool &cin, bool &cout)
{
  const double fdz      = t[td::TrdDz];
  const double pzPlusDz = p.z + fdz;
  cout                  = fabs(p.z) > (SURFACE ? fdz + kHalfTolerance : fdz);
  if (SURFACE) cin = fabs(p.z) < fdz - kHalfTolerance;
  double cross = t[td::TrdX2minusX1] * pzPlusDz - (2.0 * fdz) * (fabs(p.x) - t[td::TrdDx1]);
  if (SURFACE) {
    cout = cout || cross < -t[td::TrdTolX];
    cin  = cin && cross > t[td::TrdTolX];
  } else {
    cout = cout || cross < 0;
  }
  cross = t[td::TrdY2minusY1] * pzPlusDz - (2.0 * fdz) * (fabs(p.y) - t[td::TrdDy1]);
  if (SURFACE) {
    cout = cout || cross < -t[td::TrdTolY];
    cin  = cin && cross > t[td::TrdTolY];
  } else {
    cout = cout || cross < 0;
  }
}

__device__ __forceinline__ bool trd_contains(const double *t, D3 p)
{
  bool cin = false, cout = false;
  trd_unplaced_inside<false>(t, p, cin, cout);
  return !cout;
}

__device__ __forceinline__ int trd_inside(const double *t, D3 p)
{
  bool cin = false, cout = false;
  trd_unplaced_inside<true>(t, p, cin, cout);
  int r = kSurfaceE;
  if (cin) r = kInsideE;
  if (cout) r = kOutsideE;
  return r;
}

__device__ __forceinline__ double trd_clamp(double d) { return fabs(d) < kHalfTolerance ? 0.0 : d; }

// DistanceToIn (TrdImplementation.h:300-394)
__device__ __forceinline__ double trd_dist_in(const double *t, D3 p, D3 d)
{
  const double fdz = t[td::TrdDz];
  double distance  = kInfLength;
  const bool inz   = fabs(p.z) < fdz - kHalfTolerance;
  double distx     = t[td::TrdHalfX1plusX2] - t[td::TrdFx] * p.z;
  const bool inx   = (distx - fabs(p.x)) * t[td::TrdCalfX] > 0. + kHalfTolerance;
  const bool vary  = trd_varying_y(t);
  double disty;
  bool iny;
  if (vary) {
    disty = t[td::TrdHalfY1plusY2] - t[td::TrdFy] * p.z;
    iny   = (disty - fabs(p.y)) * t[td::TrdCalfY] > 0. + kHalfTolerance;
  } else {
    disty = fabs(p.y) - t[td::TrdDy1];
    iny   = disty < 0. - kHalfTolerance;
  }
  if (inx && iny && inz) return -1.;  // |-1| >= kHalfTolerance: no clamp
  if (p.z * d.z < 0. && !inz) {
    const double distz = (fabs(p.z) - fdz) / fabs(d.z);
    const double hitx  = fabs(p.x + distz * d.x);
    const double hity  = fabs(p.y + distz * d.y);
    const bool okzt    = p.z > (fdz - kHalfTolerance) && hitx <= t[td::TrdDx2] && hity <= t[td::TrdDy2];
    const bool okzb    = p.z < (-fdz + kHalfTolerance) && hitx <= t[td::TrdDx1] && hity <= t[td::TrdDy1];
    if (okzt || okzb) return trd_clamp(distz);
  }
  if (!inx) {
    if (trd_face<false, false, true>(t, p, d, distx)) distance = distx;
    if (trd_face<false, true, true>(t, p, d, distx)) return trd_clamp(distx);
  }
  if (vary) {
    if (!iny) {
      if (trd_face<true, false, true>(t, p, d, disty)) distance = disty;
      if (trd_face<true, true, true>(t, p, d, disty)) distance = disty;
    }
  } else if (!iny) {
    disty /= fabs(d.y);
    const double zhit = p.z + disty * d.z;
    const double xhit = p.x + disty * d.x;
    const double dx   = t[td::TrdHalfX1plusX2] - t[td::TrdFx] * zhit;
    if (p.y * d.y < 0 && disty > -kHalfTolerance && fabs(xhit) < dx && fabs(zhit) < fdz) distance = disty;
  }
  return trd_clamp(distance);
}

// DistanceToOut (TrdImplementation.h:396-499), scalar early returns
__device__ __forceinline__ double trd_dist_out(const double *t, D3 p, D3 d)
{
  const double fdz    = t[td::TrdDz];
  const double invdir = 1. / fabs(d.z + kTiny);
  bool out            = (fdz - fabs(p.z)) < 0. - kHalfTolerance;
  double distx        = t[td::TrdHalfX1plusX2] - t[td::TrdFx] * p.z;
  out                 = out || (distx - fabs(p.x)) * t[td::TrdCalfX] < 0. - kHalfTolerance;
  const bool vary     = trd_varying_y(t);
  double disty;
  if (vary) {
    disty = t[td::TrdHalfY1plusY2] - t[td::TrdFy] * p.z;
    out   = out || (disty - fabs(p.y)) * t[td::TrdCalfY] < 0. - kHalfTolerance;
  } else {
    disty = t[td::TrdDy1] - fabs(p.y);
    out   = out || disty < 0. - kHalfTolerance;
  }
  if (out) return -1.;
  if (d.z > 0.) {
    const double distz = (fdz - p.z) * invdir;
    if (fabs(p.x + distz * d.x) <= t[td::TrdDx2] && fabs(p.y + distz * d.y) <= t[td::TrdDy2]) return trd_clamp(distz);
  }
  if (d.z < 0.) {
    const double distz = (p.z + fdz) * invdir;
    if (fabs(p.x + distz * d.x) <= t[td::TrdDx1] && fabs(p.y + distz * d.y) <= t[td::TrdDy1]) return trd_clamp(distz);
  }
  if (trd_face<false, false, false>(t, p, d, distx)) return trd_clamp(distx);
  if (trd_face<false, true, false>(t, p, d, distx)) return trd_clamp(distx);
  double distance = 0.0;
  if (vary) {
    if (trd_face<true, false, false>(t, p, d, disty)) return trd_clamp(disty);
    if (trd_face<true, true, false>(t, p, d, disty)) distance = disty;
  } else {
    const double plane = d.y < 0. ? -t[td::TrdDy1] : t[td::TrdDy1];
    disty              = (plane - p.y) / d.y;
    const double zhit  = p.z + disty * d.z;
    const double xhit  = p.x + disty * d.x;
    const double dx    = t[td::TrdHalfX1plusX2] - t[td::TrdFx] * zhit;
    if (fabs(xhit) < dx && fabs(zhit) < fdz) distance = disty;
  }
  return trd_clamp(distance);
}

// ---------------------------------------------------------------- Trapezoid
// volumes/kernel/TrapezoidImplementation.h over the four side planes of
// base/PlaneShell.h (the default VECGEOM_PLANESHELL=ON build).
__device__ __forceinline__ double trap_pdist(const double *t, int i, D3 p)
{
  return t[row::TrapA + i] * p.x + t[row::TrapB + i] * p.y + t[row::TrapC + i] * p.z + t[row::TrapD + i];
}
__device__ __forceinline__ double trap_proj(const double *t, int i, D3 d)
{
  return t[row::TrapA + i] * d.x + t[row::TrapB + i] * d.y + t[row::TrapC + i] * d.z;
}

// GenericKernelForContainsAndInside (TrapezoidImplementation.h:124-162, PlaneShell.h:130-151)
template <bool FOR_INSIDE>
__device__ __forceinline__ void trap_generic_ci(const double *t, D3 p, bool &cin, bool &cout)
{
  const double dz = t[row::TrapDz];
  cout            = fabs(p.z) > (FOR_INSIDE ? dz + kHalfTolerance : dz);
  if (FOR_INSIDE) cin = fabs(p.z) < dz - kHalfTolerance;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double dist = trap_pdist(t, i, p);
    cout              = cout || dist > (FOR_INSIDE ? 0. + kHalfTolerance : 0.);
    if (FOR_INSIDE) cin = cin && dist < 0. - kHalfTolerance;
  }
}

__device__ __forceinline__ bool trap_contains(const double *t, D3 p)
{
  bool cin = false, cout = false;
  trap_generic_ci<false>(t, p, cin, cout);
  return !cout;
}

__device__ __forceinline__ int trap_inside(const double *t, D3 p)
{
  bool cin = false, cout = false;
  trap_generic_ci<true>(t, p, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// DistanceToIn (TrapezoidImplementation.h:177-216, PlaneShell.h:161-213), scalar early returns
__device__ __forceinline__ double trap_dist_in(const double *t, D3 p, D3 d)
{
  const double dz       = t[row::TrapDz];
  const double signZdir = sgn(d.z);
  const double max      = signZdir * dz - p.z;
  if (signZdir * max < 0.0 + kHalfTolerance) return kInfLength;
  const double invdir = 1.0 / nonzero(d.z);
  double smax         = max * invdir;
  double smin         = -(signZdir * dz + p.z) * invdir;
  double pdist[4], proj[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pdist[i] = trap_pdist(t, i, p);
    proj[i]  = trap_proj(t, i, d);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (pdist[i] > 0. + kHalfTolerance && proj[i] >= 0.) return kInfLength;
    if (pdist[i] > 0. - kHalfTolerance && proj[i] > 0.) return kInfLength;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double vdist     = -pdist[i] / nonzero(proj[i]);
    const bool posPoint    = pdist[i] > 0. - kHalfTolerance;
    const bool posDir      = proj[i] > 0;
    const bool fromInside  = !posPoint && posDir;
    const bool fromOutside = posPoint && !posDir;
    if (fromInside && vdist < smin) return kInfLength;
    if (fromOutside && vdist > smax) return kInfLength;
    if (fromOutside && vdist > smin) smin = vdist;
    if (fromInside && vdist < smax) smax = vdist;
  }
  return smin <= smax ? smin : kInfLength;
}

// DistanceToOut (TrapezoidImplementation.h:270-299, PlaneShell.h:219-257)
__device__ __forceinline__ double trap_dist_out(const double *t, D3 p, D3 d)
{
  const double dz = t[row::TrapDz];
  if (fabs(p.z) > dz + kHalfTolerance) return -1.0;
  double distance = kInfLength;
  if (d.z != 0.) distance = (sgn(d.z) * dz - p.z) / nonzero(d.z);
  double distOut = kInfLength;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double pdist = trap_pdist(t, i, p);
    const double proj  = trap_proj(t, i, d);
    const double vdist = -pdist / nonzero(proj);
    if (pdist > kHalfTolerance) distOut = -1.;
    if (proj > 0. && vdist < distOut) distOut = vdist;
  }
  return distOut < distance ? distOut : distance;
}

// SafetyToIn / SafetyToOut (TrapezoidImplementation.h:341-401, PlaneShell.h:260-305)
__device__ __forceinline__ double trap_safe_in(const double *t, D3 p)
{
  double safety = fabs(p.z) - t[row::TrapDz];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double dist = trap_pdist(t, i, p);
    if (dist > safety) safety = dist;
  }
  return safety;
}

__device__ __forceinline__ double trap_safe_out(const double *t, D3 p)
{
  double safety = t[row::TrapDz] - fabs(p.z);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double dist = -trap_pdist(t, i, p);
    if (dist < safety) safety = dist;
  }
  return safety;
}

// ---------------------------------------------------------------- Sphere
// volumes/kernel/SphereImplementation.h with SphereUtilities.h.  Even a full sphere
// consults its phi wedge (Wedge_Evolution.h) and theta cone (ThetaCone_Evolution.h)
// in the completely-inside/outside and on-surface tests; the full-range path below
// reproduces them for stheta = 0, etheta >= pi (what a full theta range implies), and a
// sphere with sections goes to the out-of-line sphere_sect_* functions.
namespace sp = row;
constexpr double kSqrtTolerance = 3.1622777e-5;  // base/Math.h:29
constexpr double kThetaHalfPi   = 0.5 * 3.14159265358979323846;

__device__ __forceinline__ double sph_plus_tol_sq(double x) { return x * (x + 2.0 * kTolerance); }
__device__ __forceinline__ double sph_minus_tol_sq(double x) { return fabs(x * (x - 2.0 * kTolerance)); }
__device__ __forceinline__ double mag2(D3 p) { return p.x * p.x + p.y * p.y + p.z * p.z; }

// ---------------------------------------------------------------- Sphere sections
// The general sphere (a phi range below 2 pi or a theta range short of [0, pi]): the
// full-range tests of SphereImplementation.h and SphereUtilities.h with the phi wedge's
// half-plane distances (Wedge_Evolution.h) and the theta cone (ThetaCone_Evolution.h).
// Each operation is one out-of-line function so the traversal kernels carry a call, not
// the section code, for every sphere.
constexpr double kThHalfTol = 0.5 * kTolerance;       // ThetaCone::halfAngTolerance
constexpr double kThTolAng  = 2 * kTolerance * 10.;   // ThetaCone_Evolution.h:677-747

__device__ __forceinline__ bool sph_flag(const double *t, int i) { return t[i] != 0.; }

// Wedge::IsPointOnSurfaceAndMovingOut<START, MOVING_OUT> (Wedge_Evolution.h:233-246)
template <bool START, bool MOVING_OUT>
__device__ __forceinline__ bool wedge_moving(const double *w, D3 p, D3 d)
{
  const double ax = START ? w[row::WedgeA1x] : w[row::WedgeA2x], ay = START ? w[row::WedgeA1y] : w[row::WedgeA2y];
  const double nx = START ? w[row::WedgeN1x] : w[row::WedgeN2x], ny = START ? w[row::WedgeN1y] : w[row::WedgeN2y];
  if (!wedge_on_surface(ax, ay, nx, ny, p)) return false;
  const double dn = d.x * -nx + d.y * -ny;  // dir.Dot(-normal), the normal has z = 0
  return MOVING_OUT ? dn > 0.005 * kHalfTolerance : dn < 0.005 * kHalfTolerance;
}

// Wedge::DistanceToIn / DistanceToOut (Wedge_Evolution.h:393-446)
template <bool TO_IN>
__device__ __forceinline__ void wedge_dist(const double *w, D3 p, D3 d, double &dist1, double &dist2)
{
  const double comp1 = d.x * w[row::WedgeN1x] + d.y * w[row::WedgeN1y];
  const double comp2 = d.x * w[row::WedgeN2x] + d.y * w[row::WedgeN2y];
  dist1 = kInfLength;
  dist2 = kInfLength;
  if (TO_IN ? comp1 > 0. : comp1 < 0.) {
    const double tmp = -(p.x * w[row::WedgeN1x] + p.y * w[row::WedgeN1y]) / comp1;
    if (tmp > 0.) dist1 = tmp;
  }
  if (TO_IN ? comp2 > 0. : comp2 < 0.) {
    const double tmp = -(p.x * w[row::WedgeN2x] + p.y * w[row::WedgeN2y]) / comp2;
    if (tmp > 0.) dist2 = tmp;
  }
}

__device__ __forceinline__ bool wedge_contains_p(const double *w, D3 p)
{
  bool cin = false, cout = false;
  wedge_ci<false>(w, p, cin, cout);
  return !cout;
}

// ThetaCone::IsCompletelyInside (ThetaCone_Evolution.h:655-730)
__device__ __forceinline__ bool thc_completely_inside(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double rho         = sqrt(mag2(p) - (p.z * p.z));
  const double cone1Radius = fabs(p.z * t[sp::SphTanSTheta]);
  const double cone2Radius = fabs(p.z * t[sp::SphTanETheta]);
  const bool onZ           = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool onXY          = p.z == 0. && (p.x != 0. || p.y != 0.);
  bool ci = onZ && ((sT == 0. && eT == kPiD) || (p.z > 0. && sT == 0.) || (p.z < 0. && eT == kPiD));
  ci      = ci || (!ci && (onXY && (sT < kThetaHalfPi && eT > kThetaHalfPi && (kThetaHalfPi - sT) > kTolerance &&
                                   (eT - kThetaHalfPi) > kTolerance)));
  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin = cone1Radius + kThTolAng, tolAngMax = cone2Radius - kThTolAng;
      ci = ci || (!ci && (((rho <= tolAngMax) && (rho >= tolAngMin) && (p.z > 0.) && (sT != 0.)) ||
                          ((rho <= tolAngMax) && (sT == 0.) && (p.z > 0.))));
    }
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin = cone1Radius + kThTolAng, tolAngMax = cone2Radius + kThTolAng;
      ci = ci || (!ci && (((rho >= tolAngMin) && (p.z > 0.)) || ((rho >= tolAngMax) && (p.z < 0.))));
    }
    if (eT >= kThetaHalfPi - kThHalfTol && eT <= kThetaHalfPi + kThHalfTol) ci = ci && !(fabs(p.z) < kThHalfTol);
  }
  if (eT > kThetaHalfPi + kThHalfTol) {
    if (sT >= kThetaHalfPi - kThHalfTol && sT <= kThetaHalfPi + kThHalfTol) ci = ci && !(fabs(p.z) < kThHalfTol);
    if (sT > kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin = cone1Radius - kThTolAng, tolAngMax = cone2Radius + kThTolAng;
      ci = ci || (!ci && (((rho <= tolAngMin) && (rho >= tolAngMax) && (p.z < 0.) && (eT != kPiD)) ||
                          ((rho <= tolAngMin) && (p.z < 0.) && (eT == kPiD))));
    }
  }
  return ci;
}

// ThetaCone::IsCompletelyOutside (ThetaCone_Evolution.h:733-805)
__device__ __forceinline__ bool thc_completely_outside(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double rho         = sqrt(p.x * p.x + p.y * p.y);
  const double cone1Radius = fabs(p.z * t[sp::SphTanSTheta]);
  const double cone2Radius = fabs(p.z * t[sp::SphTanETheta]);
  const bool onZ           = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool onXY          = p.z == 0. && (p.x != 0. || p.y != 0.);
  bool co = onZ && ((sT != 0. && eT != kPiD) || (p.z > 0. && sT != 0.) || (p.z < 0. && eT != kPiD));
  co      = co || (!co && (onXY && (((sT < kThetaHalfPi) && (eT < kThetaHalfPi) && ((kThetaHalfPi - sT) > kTolerance) &&
                                     ((kThetaHalfPi - eT) > kTolerance)) ||
                                    ((sT > kThetaHalfPi && eT > kThetaHalfPi) && ((sT - kThetaHalfPi) > kTolerance) &&
                                     ((eT - kThetaHalfPi) > kTolerance)))));
  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin2 = cone1Radius - kThTolAng, tolAngMax2 = cone2Radius + kThTolAng;
      co = co || (!co && ((rho < tolAngMin2) || (rho > tolAngMax2) || (p.z < 0.)));
    }
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin2 = cone1Radius - kThTolAng, tolAngMax2 = cone2Radius - kThTolAng;
      co = co || (!co && (((rho < tolAngMin2) && (p.z > 0.)) || ((rho < tolAngMax2) && (p.z < 0.))));
    }
    if (eT >= kThetaHalfPi - kThHalfTol && eT <= kThetaHalfPi + kThHalfTol) co = co && !(fabs(p.z) < kThHalfTol);
  }
  if (eT > kThetaHalfPi + kThHalfTol) {
    if (sT >= kThetaHalfPi - kThHalfTol && sT <= kThetaHalfPi + kThHalfTol) co = co && !(fabs(p.z) < kThHalfTol);
    if (sT > kThetaHalfPi + kThHalfTol && sT < eT) {
      const double tolAngMin2 = cone1Radius + kThTolAng, tolAngMax2 = cone2Radius - kThTolAng;
      co = co || (!co && ((rho < tolAngMax2) || (rho > tolAngMin2) || (p.z > 0.)));
    }
  }
  return co;
}

__device__ __forceinline__ bool thc_contains(const double *t, D3 p) { return !thc_completely_outside(t, p); }

// ThetaCone::IsPointOnSurfaceAndMovingOut<START, MOVING_OUT> (ThetaCone_Evolution.h:164-229)
template <bool START, bool MOVING_OUT>
__device__ __forceinline__ bool thc_moving(const double *t, D3 p, D3 d)
{
  const double rhs  = fabs(t[START ? sp::SphTanSTheta : sp::SphTanETheta] * p.z);
  const double rho2 = p.x * p.x + p.y * p.y;
  if (!(rho2 >= sph_minus_tol_sq(rhs) && rho2 <= sph_plus_tol_sq(rhs))) return false;
  D3 n{p.x, p.y, -t[START ? sp::SphTanSTheta2 : sp::SphTanETheta2] * p.z};
  if (START ? t[sp::SphSTheta] <= kThetaHalfPi : !(t[sp::SphETheta] <= kThetaHalfPi)) n = D3{-n.x, -n.y, -n.z};
  const double dn = d.x * n.x + d.y * n.y + d.z * n.z;
  return MOVING_OUT ? dn > 0. : dn < 0.;
}

// ThetaCone::DistanceToLine (ThetaCone_Evolution.h:358-365)
__device__ __forceinline__ double thc_dist_line(double slope, double x, double y)
{
  const double dist = (y - slope * x) / sqrt(1. + slope * slope);
  return fabs(dist);
}

// ThetaCone::SafetyToIn (ThetaCone_Evolution.h:276-316)
__device__ __forceinline__ double thc_safe_in(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double pointRad = sqrt(p.x * p.x + p.y * p.y);
  const double sfTh1    = thc_dist_line(t[sp::SphSlope1], pointRad, p.z);
  const double sfTh2    = thc_dist_line(t[sp::SphSlope2], pointRad, p.z);
  double safeTheta      = vmin(sfTh1, sfTh2);
  if (thc_contains(t, p)) return 0.;
  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT && p.z < 0.) safeTheta = sfTh2;
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
      if (p.z > 0.) safeTheta = sfTh1;
      if (p.z < 0.) safeTheta = sfTh2;
    }
  }
  if (eT > kThetaHalfPi + kThHalfTol && sT > kThetaHalfPi + kThHalfTol && sT < eT && p.z > 0.) safeTheta = sfTh1;
  return safeTheta;
}

// ThetaCone::SafetyToOut (ThetaCone_Evolution.h:318-356)
__device__ __forceinline__ double thc_safe_out(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double pointRad    = sqrt(p.x * p.x + p.y * p.y);
  const double bisectorRad = fabs(p.z * t[sp::SphTanBisector]);
  bool cond                = false;
  const double sfTh1       = thc_dist_line(t[sp::SphSlope1], pointRad, p.z);
  const double sfTh2       = thc_dist_line(t[sp::SphSlope2], pointRad, p.z);
  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT) cond = (pointRad < bisectorRad) && (sT != 0.);
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) cond = sfTh1 < sfTh2;
  }
  if (eT > kThetaHalfPi + kThHalfTol && sT > kThetaHalfPi + kThHalfTol && sT < eT)
    cond = !((pointRad < bisectorRad) && (eT != kPiD));
  return cond ? sfTh1 : sfTh2;
}

// ThetaCone::DistanceToIn's root clean-up (ThetaCone_Evolution.h:387-395)
__device__ __forceinline__ double thc_in_root(double root, bool &done)
{
  done = done || (fabs(root) < 3. * kTolerance);
  if (fabs(root) < 3. * kTolerance) root = 0.;
  if (!done && root < 0.) root = kInfLength;
  return root;
}

// ThetaCone::DistanceToIn (ThetaCone_Evolution.h:367-496); dist1/dist2 and int1/int2 come
// in as kInfLength and false
__device__ __forceinline__ void thc_dist_in(const double *t, D3 p, D3 d, double &dist1, double &dist2, bool &int1,
                                            bool &int2)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double tanS2 = t[sp::SphTanSTheta2], tanE2 = t[sp::SphTanETheta2];
  bool done          = false;
  double firstRoot = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = p.x * d.x + p.y * d.y;
  const double rho2    = p.x * p.x + p.y * p.y;
  const double dirRho2 = d.x * d.x + d.y * d.y;
  const double b       = pDotV2d - p.z * d.z * tanS2;
  const double a       = dirRho2 - d.z * d.z * tanS2;
  const double cc      = rho2 - p.z * p.z * tanS2;
  const double d2      = b * b - a * cc;
  const double aInv    = 1. / nonzero(a);
  if (d2 > 0.) firstRoot = (-b + sqrt(fabs(d2))) * aInv;
  firstRoot = thc_in_root(firstRoot, done);

  const double b2    = pDotV2d - p.z * d.z * tanE2;
  const double a2    = dirRho2 - d.z * d.z * tanE2;
  const double c2    = rho2 - p.z * p.z * tanE2;
  const double d22   = b2 * b2 - a2 * c2;
  const double a2Inv = 1. / nonzero(a2);
  if (d22 > 0.) secondRoot = (-b2 - sqrt(fabs(d22))) * a2Inv;
  if (!done && fabs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
  done = done || (fabs(secondRoot) < 3. * kTolerance);
  if (!done && secondRoot < 0.) secondRoot = kInfLength;

  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT) {
      dist1 = firstRoot;
      dist2 = secondRoot;
      const double z1 = (p.z + dist1 * d.z), z2 = (p.z + dist2 * d.z);
      int1 = ((d2 > 0.) && (z1 > 0.));
      int2 = ((d22 > 0.) && (z2 > 0.));
    }
    if (eT >= kThetaHalfPi - kThHalfTol && eT <= kThetaHalfPi + kThHalfTol) {
      if (d.z > 0.) dist2 = -p.z / d.z;
      const double z2 = (p.z + dist2 * d.z);
      int2 = ((dist2 != kInfLength) && (fabs(z2) < kThHalfTol));
    }
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
      dist1 = firstRoot;
      if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
      done       = false;
      secondRoot = thc_in_root(secondRoot, done);
      dist2      = secondRoot;
      const double z1 = (p.z + dist1 * d.z), z2 = (p.z + dist2 * d.z);
      int1 = ((d2 > 0) && (dist1 != kInfLength) && (z1 > 0.));
      int2 = ((d22 > 0) && (dist2 != kInfLength) && (z2 < 0.));
    }
  }
  if (sT >= kThetaHalfPi - kThHalfTol && eT > kThetaHalfPi + kThHalfTol && sT < eT) {
    if (d2 > 0.) firstRoot = (-b - sqrt(fabs(d2))) * aInv;
    done      = false;
    firstRoot = thc_in_root(firstRoot, done);
    dist1     = firstRoot;
    if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
    done       = false;
    secondRoot = thc_in_root(secondRoot, done);
    dist2      = secondRoot;
    const double z1 = (p.z + dist1 * d.z), z2 = (p.z + dist2 * d.z);
    int1 = ((d2 > 0) && (dist1 != kInfLength) && (z1 < 0.));
    int2 = ((d22 > 0) && (dist2 != kInfLength) && (z2 < 0.));
  }
  if (sT >= kThetaHalfPi - kThHalfTol && sT <= kThetaHalfPi + kThHalfTol) {
    if (d.z < 0.) dist1 = -p.z / d.z;
    const double z1 = (p.z + dist1 * d.z);
    int1 = ((dist1 != kInfLength) && (fabs(z1) < kThHalfTol));
  }
}

// ThetaCone::DistanceToOut (ThetaCone_Evolution.h:498-652), same conventions
__device__ __forceinline__ void thc_dist_out(const double *t, D3 p, D3 d, double &dist1, double &dist2, bool &int1,
                                             bool &int2)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double tanS2 = t[sp::SphTanSTheta2], tanE2 = t[sp::SphTanETheta2];
  double firstRoot = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = p.x * d.x + p.y * d.y;
  const double rho2    = p.x * p.x + p.y * p.y;
  const double b       = pDotV2d - p.z * d.z * tanS2;
  const double a       = d.x * d.x + d.y * d.y - d.z * d.z * tanS2;
  const double cc      = rho2 - p.z * p.z * tanS2;
  double d2            = b * b - a * cc;
  if (d2 < 0. && fabs(d2) < kHalfTolerance) d2 = 0.;
  if ((d2 >= 0.) && b >= 0. && a != 0.) firstRoot = ((-b - sqrt(fabs(d2))) / nonzero(a));
  if ((d2 >= 0.) && b < 0.) firstRoot = ((cc) / nonzero(-b + sqrt(fabs(d2))));
  if (firstRoot < 0.) firstRoot = kInfLength;

  const double b2 = p.x * d.x + p.y * d.y - p.z * d.z * tanE2;
  const double a2 = d.x * d.x + d.y * d.y - d.z * d.z * tanE2;
  const double c2 = p.x * p.x + p.y * p.y - p.z * p.z * tanE2;
  double d22      = (b2 * b2) - (a2 * c2);
  if (d22 < 0. && fabs(d22) < kHalfTolerance) d22 = 0.;
  if ((d22 >= 0.) && b2 >= 0.) secondRoot = ((c2) / nonzero(-b2 - sqrt(fabs(d22))));
  if ((d22 >= 0.) && b2 < 0. && a2 != 0.) secondRoot = ((-b2 + sqrt(fabs(d22))) / nonzero(a2));
  if (secondRoot < 0. && fabs(secondRoot) > kTolerance) secondRoot = kInfLength;
  if (fabs(secondRoot) < kTolerance) secondRoot = 0.;

  if (sT < kThetaHalfPi + kThHalfTol) {
    if (eT < kThetaHalfPi + kThHalfTol && sT < eT) {
      dist1 = firstRoot;
      dist2 = secondRoot;
      const double z1 = (p.z + dist1 * d.z), z2 = (p.z + dist2 * d.z);
      int1 = ((d2 > 0) && (dist1 != kInfLength) && ((z1) > -kHalfTolerance));
      int2 = ((d22 > 0) && (dist2 != kInfLength) && ((z2) > -kHalfTolerance));
      const double dirRho2 = d.x * d.x + d.y * d.y;
      double zs = kInfLength, ze = kInfLength;
      if (sT != 0.) zs = dirRho2 / t[sp::SphTanSTheta];
      if (eT != 0.) ze = dirRho2 / t[sp::SphTanETheta];
      const bool cond = (p.x == 0. && p.y == 0. && p.z == 0. && d.z < zs && d.z < ze);
      if (cond) dist1 = 0.;
      if (cond) dist2 = 0.;
      int1 = int1 || cond;
      int2 = int2 || cond;
    }
    if (eT >= kThetaHalfPi - kThHalfTol && eT <= kThetaHalfPi + kThHalfTol) {
      dist1 = firstRoot;
      dist2 = kInfLength;
      if (d.z < 0.) dist2 = -1. * p.z / d.z;
      const double z2 = (p.z + dist2 * d.z), z1 = (p.z + dist1 * d.z);
      int2 = ((dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && !(d.z == 0.));
      int1 = ((d2 >= 0) && (dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && !(d.z == 0.));
    }
    if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
      dist1 = firstRoot;
      if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / nonzero(a2));
      if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / nonzero(-b2 + sqrt(fabs(d22))));
      if (secondRoot < 0.) secondRoot = kInfLength;
      dist2 = secondRoot;
      const double z1 = (p.z + dist1 * d.z), z2 = (p.z + dist2 * d.z);
      int1 = ((d2 >= 0) && (dist1 != kInfLength) && ((z1) > -kHalfTolerance));
      int2 = ((d22 >= 0) && (dist2 != kInfLength) && ((z2) < kHalfTolerance));
    }
  }
  if (eT > kThetaHalfPi + kThHalfTol && sT < eT) {
    secondRoot = kInfLength;
    if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / nonzero(a2));
    if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / nonzero(-b2 + sqrt(fabs(d22))));
    dist2 = secondRoot;
    if (sT > kThetaHalfPi + kThHalfTol) {
      if ((d2 >= 0.) && b > 0.) firstRoot = ((cc) / nonzero(-b - sqrt(fabs(d2))));
      if ((d2 >= 0.) && b <= 0. && a != 0.) firstRoot = ((-b + sqrt(fabs(d2))) / nonzero(a));
      if (firstRoot < 0.) firstRoot = kInfLength;
      dist1           = firstRoot;
      const double z1 = (p.z + dist1 * d.z);
      int1            = ((d2 > 0) && (dist1 != kInfLength) && ((z1) < kHalfTolerance));
      const double z2 = (p.z + dist2 * d.z);
      int2            = ((d22 > 0) && (dist2 != kInfLength) && ((z2) < kHalfTolerance));
      const double dirRho2 = d.x * d.x + d.y * d.y;
      double zs = -kInfLength, ze = -kInfLength;
      if (t[sp::SphTanSTheta] != 0.) zs = -dirRho2 / t[sp::SphTanSTheta];
      if (t[sp::SphTanETheta] != 0.) ze = -dirRho2 / t[sp::SphTanETheta];
      const bool cond = (p.x == 0. && p.y == 0. && p.z == 0. && d.z > zs && d.z > ze);
      if (cond) dist1 = 0.;
      if (cond) dist2 = 0.;
      int1 = int1 || cond;
      int2 = int2 || cond;
    }
  }
  if (sT >= kThetaHalfPi - kThHalfTol && sT <= kThetaHalfPi + kThHalfTol) {
    dist2 = secondRoot;
    dist1 = kInfLength;
    if (d.z > 0.) dist1 = -1. * p.z / nonzero(d.z);
    const double z1 = (p.z + dist1 * d.z);
    const double z2 = (p.z + dist2 * d.z);
    int1 = ((dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && (d.z != 0.));
    int2 = ((d22 >= 0) && (dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && (d.z != 0.));
  }
}

// SphereUtilities::IsCompletelyInside / IsCompletelyOutside (SphereUtilities.h:110-141)
__device__ __forceinline__ bool sphs_completely_inside(const double *t, D3 p)
{
  const double rad = sqrt(mag2(p));
  const bool inRad = (rad < (t[sp::SphRmax] - kTolerance)) && (rad > (t[sp::SphRmin] + kTolerance));
  bool cin = false, cout = false;
  wedge_ci<true>(t + sp::SphA1x, p, cin, cout);
  return inRad && cin && thc_completely_inside(t, p);
}

__device__ __forceinline__ bool sphs_completely_outside(const double *t, D3 p)
{
  const double rad  = sqrt(mag2(p));
  const bool outRad = (rad > (t[sp::SphRmax] + kTolerance)) || (rad < (t[sp::SphRmin] - kTolerance));
  bool cin = false, cout = false;
  wedge_ci<true>(t + sp::SphA1x, p, cin, cout);
  return outRad || cout || thc_completely_outside(t, p);
}

// SphereUtilities::IsPointOnSurfaceAndMovingOut (SphereUtilities.h:143-195)
template <bool MOVING_OUT>
__device__ __forceinline__ bool sphs_on_surface_moving(const double *t, D3 p, D3 d)
{
  const double m2   = mag2(p);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double dp   = d.x * p.x + d.y * p.y + d.z * p.z;
  const bool outer  = (m2 <= sph_plus_tol_sq(rmax) && m2 >= sph_minus_tol_sq(rmax)) &&
                     (MOVING_OUT ? dp > kSqrtTolerance : dp < -kSqrtTolerance);
  bool inner = false;
  if (rmin != 0.) {
    const double dmp = d.x * -p.x + d.y * -p.y + d.z * -p.z;
    inner            = (m2 <= sph_plus_tol_sq(rmin) && m2 >= sph_minus_tol_sq(rmin)) &&
            (MOVING_OUT ? dmp > kSqrtTolerance : dmp < -kSqrtTolerance);
  }
  const double *w = t + sp::SphA1x;
  bool phiFace = false, thetaFace = false;
  if (t[sp::SphDPhi] < (2. * kPiD - kHalfTolerance))
    phiFace = wedge_moving<true, MOVING_OUT>(w, p, d) || wedge_moving<false, MOVING_OUT>(w, p, d);
  if (t[sp::SphDTheta] < (kPiD - kHalfTolerance))
    thetaFace = thc_moving<true, MOVING_OUT>(t, p, d) || thc_moving<false, MOVING_OUT>(t, p, d);
  const bool inShell = (m2 >= rmin * rmin) && (m2 <= rmax * rmax);
  return ((outer || inner) && wedge_contains_p(w, p) && thc_contains(t, p)) ||
         (phiFace && inShell && thc_contains(t, p)) || (thetaFace && inShell && wedge_contains_p(w, p));
}

// SphereImplementation::GenericKernelForContainsAndInside<FOR_INSIDE> (SphereImplementation.h:89-136)
template <bool FOR_INSIDE>
__device__ __forceinline__ void sphs_ci(const double *t, D3 p, bool &cin, bool &cout)
{
  const double rad2 = mag2(p);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  if (rmin != 0.) {
    cin  = rad2 <= sph_minus_tol_sq(rmax) && rad2 >= sph_plus_tol_sq(rmin);
    cout = rad2 >= sph_plus_tol_sq(rmax) || rad2 <= sph_minus_tol_sq(rmin);
  } else {
    cin  = rad2 <= sph_minus_tol_sq(rmax);
    cout = rad2 >= sph_plus_tol_sq(rmax);
  }
  if (!sph_flag(t, sp::SphFullPhi)) {
    bool ci = false, co = false;
    wedge_ci<FOR_INSIDE>(t + sp::SphA1x, p, ci, co);
    cout = cout || co;
    if (FOR_INSIDE) cin = cin && ci;
  }
  if (!sph_flag(t, sp::SphFullTheta)) {
    const bool ci = FOR_INSIDE ? thc_completely_inside(t, p) : false;
    const bool co = thc_completely_outside(t, p);
    cout          = cout || co;
    if (FOR_INSIDE) cin = cin && ci;
  }
}

// SphereImplementation::GetMinDistFromPhi<TO_IN> (SphereImplementation.h:343-386)
template <bool TO_IN>
__device__ __forceinline__ void sphs_min_dist_phi(const double *t, D3 p, D3 d, double &distance)
{
  const double *w = t + sp::SphA1x;
  const double rmin2 = t[sp::SphRmin] * t[sp::SphRmin], rmax2 = t[sp::SphRmax] * t[sp::SphRmax];
  double distPhi1, distPhi2;
  wedge_dist<TO_IN>(w, p, d, distPhi1, distPhi2);
  double dist = vmin(distPhi1, distPhi2);
  D3 tmp{p.x + dist * d.x, p.y + dist * d.y, p.z + dist * d.z};
  double rad2 = mag2(tmp);
  bool onFace = ((dist == distPhi1) && wedge_on_surface(w[row::WedgeA1x], w[row::WedgeA1y], w[row::WedgeN1x],
                                                         w[row::WedgeN1y], tmp)) ||
                ((dist == distPhi2) && wedge_on_surface(w[row::WedgeA2x], w[row::WedgeA2y], w[row::WedgeN2x],
                                                         w[row::WedgeN2y], tmp));
  const bool cond1 = onFace && (rad2 > rmin2) && (rad2 < rmax2) && thc_contains(t, tmp);
  if (cond1) distance = vmin(dist, distance);
  dist   = vmax(distPhi1, distPhi2);
  tmp    = D3{p.x + dist * d.x, p.y + dist * d.y, p.z + dist * d.z};
  rad2   = mag2(tmp);
  onFace = ((dist == distPhi1) && wedge_on_surface(w[row::WedgeA1x], w[row::WedgeA1y], w[row::WedgeN1x],
                                                    w[row::WedgeN1y], tmp)) ||
           ((dist == distPhi2) && wedge_on_surface(w[row::WedgeA2x], w[row::WedgeA2y], w[row::WedgeN2x],
                                                    w[row::WedgeN2y], tmp));
  const bool cond2 = onFace && (rad2 > rmin2) && (rad2 < rmax2) && thc_contains(t, tmp);
  if (!cond1 && cond2) distance = vmin(dist, distance);
}

// DistanceToIn (SphereImplementation.h:138-256) of a sphere with sections
__device__ __noinline__ double sphere_sect_dist_in(const double *t, D3 p, D3 d)
{
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double *w      = t + sp::SphA1x;
  const double rad2    = mag2(p);
  const double pDotV3d = p.x * d.x + p.y * d.y + p.z * d.z;
  double c             = rad2 - rmax * rmax;
  if (sphs_completely_inside(t, p)) return -1.0;
  if (sphs_on_surface_moving<false>(t, p, d)) return 0.0;
  double d2 = (pDotV3d * pDotV3d - c);
  if (d2 < 0. || ((c > 0.) && (pDotV3d > 0.))) return kInfLength;
  double sd1 = kInfLength, sd2 = kInfLength;
  if (d2 >= 0.) sd1 = (-pDotV3d - sqrt(fabs(d2)));
  double outerDist = kInfLength, innerDist = kInfLength;
  {
    const D3 tmp{p.x + sd1 * d.x, p.y + sd1 * d.y, p.z + sd1 * d.z};
    if (wedge_contains_p(w, tmp) && thc_contains(t, tmp) && (sd1 >= 0.)) outerDist = sd1;
  }
  if (rmin != 0.) {
    c  = rad2 - rmin * rmin;
    d2 = pDotV3d * pDotV3d - c;
    if (d2 >= 0.) sd2 = (-pDotV3d + sqrt(fabs(d2)));
    const D3 tmp{p.x + sd2 * d.x, p.y + sd2 * d.y, p.z + sd2 * d.z};
    if ((sd2 >= 0.) && wedge_contains_p(w, tmp) && thc_contains(t, tmp)) innerDist = sd2;
  }
  double distance = vmin(outerDist, innerDist);
  if (!sph_flag(t, sp::SphFullPhi)) sphs_min_dist_phi<true>(t, p, d, distance);
  double distThetaMin = kInfLength;
  if (!sph_flag(t, sp::SphFullTheta)) {
    bool int1 = false, int2 = false;
    double dt1 = kInfLength, dt2 = kInfLength;
    thc_dist_in(t, p, d, dt1, dt2, int1, int2);
    const D3 c1{p.x + dt1 * d.x, p.y + dt1 * d.y, p.z + dt1 * d.z};
    const D3 c2{p.x + dt2 * d.x, p.y + dt2 * d.y, p.z + dt2 * d.z};
    const double r1 = mag2(c1), r2 = mag2(c2);
    bool valid1 = (r1 >= rmin * rmin && r1 <= rmax * rmax) && int1;
    bool valid2 = (r2 >= rmin * rmin && r2 <= rmax * rmax) && int2;
    if (!sph_flag(t, sp::SphFullPhi)) {
      valid1 = valid1 && wedge_contains_p(w, c1);
      valid2 = valid2 && wedge_contains_p(w, c2);
    }
    if (valid2 && !valid1) distThetaMin = dt2;
    if (valid1 && !valid2) distThetaMin = dt1;
    if (valid1 && valid2) distThetaMin = vmin(dt1, dt2);
  }
  distance = vmin(distThetaMin, distance);
  // a ray aimed at the centre of a theta section enters at the apex
  const D3 toC         = {0. - p.x, 0. - p.y, 0. - p.z};
  const double m2      = mag2(toC);
  const double newDist = sqrt(m2);
  const double un      = sqrt(m2 + 2.2250738585072014e-308);  // Vector3D::Unit: / Sqrt(mag2 + kMinimum)
  if ((t[sp::SphSTheta] > kHalfTolerance || t[sp::SphEThetaChk] < (kPiD - kHalfTolerance)) &&
      (fabs(toC.x / un - d.x) < kHalfTolerance) && (fabs(toC.y / un - d.y) < kHalfTolerance) &&
      (fabs(toC.z / un - d.z) < kHalfTolerance))
    distance = vmin(distance, newDist);
  return distance;
}

// DistanceToOut (SphereImplementation.h:258-341) of a sphere with sections
__device__ __noinline__ double sphere_sect_dist_out(const double *t, D3 p, D3 d)
{
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double pDotV3d = p.x * d.x + p.y * d.y + p.z * d.z;
  const double rad2    = mag2(p);
  double c             = rad2 - rmax * rmax;
  if (sphs_completely_outside(t, p)) return -1.0;
  if (sphs_on_surface_moving<true>(t, p, d)) return 0.0;
  double d2  = (pDotV3d * pDotV3d - c);
  double sd1 = kInfLength, sd2 = kInfLength;
  if (d2 >= 0.) sd1 = (-pDotV3d + sqrt(fabs(d2)));
  if (rmin != 0.) {
    c  = rad2 - rmin * rmin;
    d2 = (pDotV3d * pDotV3d - c);
    if ((d2 >= 0.) && (pDotV3d < 0.)) sd2 = (-pDotV3d - sqrt(fabs(d2)));
  }
  const double snxt = vmin(sd1, sd2);
  const double sT = t[sp::SphSTheta], eTc = t[sp::SphEThetaChk];
  const bool condSemi = ((sT == 0. && eTc == kPiD / 2.) && d.z >= 0.) || ((sT == kPiD / 2. && eTc == kPiD) && d.z <= 0.);
  if (condSemi) return snxt;
  double distThetaMin = kInfLength;
  if (!sph_flag(t, sp::SphFullTheta)) {
    bool int1 = false, int2 = false;
    double dt1 = kInfLength, dt2 = kInfLength;
    thc_dist_out(t, p, d, dt1, dt2, int1, int2);
    if (int2 && !int1) distThetaMin = dt2;
    if (!int2 && int1) distThetaMin = dt1;
    if (int2 && int1) distThetaMin = vmin(dt1, dt2);
  }
  double distance = vmin(distThetaMin, snxt);
  if (!sph_flag(t, sp::SphFullPhi)) {
    if (t[sp::SphDPhi] <= kPiD) {
      double dp1, dp2;
      wedge_dist<false>(t + sp::SphA1x, p, d, dp1, dp2);
      distance = vmin(vmin(dp1, dp2), distance);
    } else {
      sphs_min_dist_phi<false>(t, p, d, distance);
    }
  }
  return distance;
}

// SafetyToIn / SafetyToOut (SphereImplementation.h:388-479) of a sphere with sections
__device__ __noinline__ double sphere_sect_safe_in(const double *t, D3 p)
{
  const double rad = sqrt(mag2(p));
  bool cin = false, cout = false;
  sphs_ci<true>(t, p, cin, cout);
  if (cin) return -1.0;
  if (!cout) return 0.0;
  double safety;
  if (t[sp::SphRmin] != 0.) {
    const double safeRMin = t[sp::SphRmin] - rad;
    const double safeRMax = rad - t[sp::SphRmax];
    safety                = safeRMin > safeRMax ? safeRMin : safeRMax;
  } else {
    safety = rad - t[sp::SphRmax];
  }
  if (!sph_flag(t, sp::SphFullPhi)) safety = vmax(wedge_safe_in(t + sp::SphA1x, p), safety);
  if (!sph_flag(t, sp::SphFullTheta)) safety = vmax(thc_safe_in(t, p), safety);
  return safety;
}

__device__ __noinline__ double sphere_sect_safe_out(const double *t, D3 p)
{
  const double rad = sqrt(mag2(p));
  bool cin = false, cout = false;
  sphs_ci<true>(t, p, cin, cout);
  if (cout) return -1.0;
  if (!cin) return 0.0;
  double safety;
  if (t[sp::SphRmin] != 0.) {
    const double safeRMin = (rad - t[sp::SphRmin]);
    const double safeRMax = (t[sp::SphRmax] - rad);
    safety                = safeRMin < safeRMax ? safeRMin : safeRMax;
  } else {
    safety = t[sp::SphRmax] - rad;
  }
  if (!sph_flag(t, sp::SphFullPhi)) safety = vmin(wedge_safe_out(t + sp::SphA1x, p), safety);
  if (!sph_flag(t, sp::SphFullTheta)) safety = vmin(thc_safe_out(t, p), safety);
  return safety;
}

// Contains / Inside (SphereImplementation.h:62-87) of a sphere with sections
__device__ __noinline__ int sphere_sect_inside(const double *t, D3 p, bool for_contains)
{
  bool cin = false, cout = false;
  if (for_contains) {
    sphs_ci<false>(t, p, cin, cout);
    return !cout;
  }
  sphs_ci<true>(t, p, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// ---------------------------------------------------------------- Sphere (full ranges)


// ThetaCone::IsCompletelyInside (ThetaCone_Evolution.h:655-730), stheta = 0 and etheta >= pi
__device__ __forceinline__ bool theta_completely_inside(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double rho         = sqrt(mag2(p) - (p.z * p.z));
  const double cone1Radius = fabs(p.z * t[sp::SphTanSTheta]);
  const double cone2Radius = fabs(p.z * t[sp::SphTanETheta]);
  const bool onZ           = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool onXY          = p.z == 0. && (p.x != 0. || p.y != 0.);
  bool ci = onZ && ((sT == 0. && eT == kPiD) || (p.z > 0. && sT == 0.) || (p.z < 0. && eT == kPiD));
  ci      = ci || (!ci && (onXY && (sT < kThetaHalfPi && eT > kThetaHalfPi && (kThetaHalfPi - sT) > kTolerance &&
                                   (eT - kThetaHalfPi) > kTolerance)));
  const double tolAngMin = cone1Radius + 2 * kTolerance * 10.;
  const double tolAngMax = cone2Radius + 2 * kTolerance * 10.;
  return ci || (!ci && ((rho >= tolAngMin && p.z > 0.) || (rho >= tolAngMax && p.z < 0.)));
}

// ThetaCone::IsCompletelyOutside (ThetaCone_Evolution.h:733-805), stheta = 0 and etheta >= pi
__device__ __forceinline__ bool theta_completely_outside(const double *t, D3 p)
{
  const double sT = t[sp::SphSTheta], eT = t[sp::SphETheta];
  const double rho         = sqrt(p.x * p.x + p.y * p.y);
  const double cone1Radius = fabs(p.z * t[sp::SphTanSTheta]);
  const double cone2Radius = fabs(p.z * t[sp::SphTanETheta]);
  const bool onZ           = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool co = onZ && ((sT != 0. && eT != kPiD) || (p.z > 0. && sT != 0.) || (p.z < 0. && eT != kPiD));
  const double tolAngMin2 = cone1Radius - 2 * kTolerance * 10.;
  const double tolAngMax2 = cone2Radius - 2 * kTolerance * 10.;
  return co || (!co && ((rho < tolAngMin2 && p.z > 0.) || (rho < tolAngMax2 && p.z < 0.)));
}

// SphereUtilities::IsCompletelyInside / IsCompletelyOutside (SphereUtilities.h:110-141)
__device__ __forceinline__ bool sphere_completely_inside(const double *t, D3 p)
{
  const double rad   = sqrt(mag2(p));
  const bool inRad   = (rad < (t[sp::SphRmax] - kTolerance)) && (rad > (t[sp::SphRmin] + kTolerance));
  bool cin = false, cout = false;
  wedge_ci<true>(t + sp::SphA1x, p, cin, cout);
  return inRad && cin && theta_completely_inside(t, p);
}

__device__ __forceinline__ bool sphere_completely_outside(const double *t, D3 p)
{
  const double rad  = sqrt(mag2(p));
  const bool outRad = (rad > (t[sp::SphRmax] + kTolerance)) || (rad < (t[sp::SphRmin] - kTolerance));
  bool cin = false, cout = false;
  wedge_ci<true>(t + sp::SphA1x, p, cin, cout);
  return outRad || cout || theta_completely_outside(t, p);
}

// SphereUtilities::IsPointOnSurfaceAndMovingOut (SphereUtilities.h:143-195), radial faces only
template <bool MOVING_OUT>
__device__ __forceinline__ bool sphere_on_surface_moving(const double *t, D3 p, D3 d)
{
  const double m2   = mag2(p);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double dp   = d.x * p.x + d.y * p.y + d.z * p.z;
  const bool outer  = (m2 <= sph_plus_tol_sq(rmax) && m2 >= sph_minus_tol_sq(rmax)) &&
                     (MOVING_OUT ? dp > kSqrtTolerance : dp < -kSqrtTolerance);
  bool inner = false;
  if (rmin != 0.) {
    const double dmp = d.x * -p.x + d.y * -p.y + d.z * -p.z;
    inner            = (m2 <= sph_plus_tol_sq(rmin) && m2 >= sph_minus_tol_sq(rmin)) &&
            (MOVING_OUT ? dmp > kSqrtTolerance : dmp < -kSqrtTolerance);
  }
  if (!(outer || inner)) return false;
  bool cin = false, cout = false;
  wedge_ci<false>(t + sp::SphA1x, p, cin, cout);
  return !cout && !theta_completely_outside(t, p);
}

// SphereImplementation::GenericKernelForContainsAndInside (SphereImplementation.h:89-136)
__device__ __forceinline__ void sphere_ci(const double *t, D3 p, bool &cin, bool &cout)
{
  const double rad2 = mag2(p);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  if (rmin != 0.) {
    cin  = rad2 <= sph_minus_tol_sq(rmax) && rad2 >= sph_plus_tol_sq(rmin);
    cout = rad2 >= sph_plus_tol_sq(rmax) || rad2 <= sph_minus_tol_sq(rmin);
  } else {
    cin  = rad2 <= sph_minus_tol_sq(rmax);
    cout = rad2 >= sph_plus_tol_sq(rmax);
  }
}

__device__ __forceinline__ bool sphere_contains(const double *t, D3 p)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_inside(t, p, true);
  bool cin = false, cout = false;
  sphere_ci(t, p, cin, cout);
  return !cout;
}

__device__ __forceinline__ int sphere_inside(const double *t, D3 p)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_inside(t, p, false);
  bool cin = false, cout = false;
  sphere_ci(t, p, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// DistanceToIn (SphereImplementation.h:138-256), full sphere
__device__ __forceinline__ double sphere_dist_in(const double *t, D3 p, D3 d)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_dist_in(t, p, d);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double rad2    = mag2(p);
  const double pDotV3d = p.x * d.x + p.y * d.y + p.z * d.z;
  double c             = rad2 - rmax * rmax;
  if (sphere_completely_inside(t, p)) return -1.0;
  if (sphere_on_surface_moving<false>(t, p, d)) return 0.0;
  double d2 = (pDotV3d * pDotV3d - c);
  if (d2 < 0. || ((c > 0.) && (pDotV3d > 0.))) return kInfLength;
  double outerDist = kInfLength, innerDist = kInfLength;
  const double sd1 = d2 >= 0. ? (-pDotV3d - sqrt(fabs(d2))) : kInfLength;
  if (sd1 >= 0.) outerDist = sd1;
  if (rmin != 0.) {
    c                = rad2 - rmin * rmin;
    d2               = pDotV3d * pDotV3d - c;
    const double sd2 = d2 >= 0. ? (-pDotV3d + sqrt(fabs(d2))) : kInfLength;
    if (sd2 >= 0.) innerDist = sd2;
  }
  return vmin(kInfLength, vmin(outerDist, innerDist));
}

// DistanceToOut (SphereImplementation.h:258-341), full sphere
__device__ __forceinline__ double sphere_dist_out(const double *t, D3 p, D3 d)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_dist_out(t, p, d);
  const double rmax = t[sp::SphRmax], rmin = t[sp::SphRmin];
  const double pDotV3d = p.x * d.x + p.y * d.y + p.z * d.z;
  const double rad2    = mag2(p);
  double c             = rad2 - rmax * rmax;
  if (sphere_completely_outside(t, p)) return -1.0;
  if (sphere_on_surface_moving<true>(t, p, d)) return 0.0;
  double d2        = (pDotV3d * pDotV3d - c);
  const double sd1 = d2 >= 0. ? (-pDotV3d + sqrt(fabs(d2))) : kInfLength;
  double sd2       = kInfLength;
  if (rmin != 0.) {
    c  = rad2 - rmin * rmin;
    d2 = (pDotV3d * pDotV3d - c);
    if ((d2 >= 0.) && (pDotV3d < 0.)) sd2 = (-pDotV3d - sqrt(fabs(d2)));
  }
  return vmin(kInfLength, vmin(sd1, sd2));
}

// SafetyToIn / SafetyToOut (SphereImplementation.h:388-479), full sphere
__device__ __forceinline__ double sphere_safe_in(const double *t, D3 p)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_safe_in(t, p);
  const double rad = sqrt(mag2(p));
  bool cin = false, cout = false;
  sphere_ci(t, p, cin, cout);
  if (cin) return -1.0;
  if (!cout) return 0.0;
  if (t[sp::SphRmin] != 0.) {
    const double safeRMin = t[sp::SphRmin] - rad;
    const double safeRMax = rad - t[sp::SphRmax];
    return safeRMin > safeRMax ? safeRMin : safeRMax;
  }
  return rad - t[sp::SphRmax];
}

__device__ __forceinline__ double sphere_safe_out(const double *t, D3 p)
{
  if (VGN_SECTIONS && !sph_flag(t, sp::SphFull)) return sphere_sect_safe_out(t, p);
  const double rad = sqrt(mag2(p));
  bool cin = false, cout = false;
  sphere_ci(t, p, cin, cout);
  if (cout) return -1.0;
  if (!cin) return 0.0;
  if (t[sp::SphRmin] != 0.) {
    const double safeRMin = (rad - t[sp::SphRmin]);
    const double safeRMax = (t[sp::SphRmax] - rad);
    return safeRMin < safeRMax ? safeRMin : safeRMax;
  }
  return t[sp::SphRmax] - rad;
}

// ---------------------------------------------------------------- Polycone
// volumes/kernel/PolyconeImplementation.h over the sections' cone rows.  The kernels have
// no phi logic of their own: a phi section reaches them through its section cones (built
// with the polycone's raw phi arguments, PolyconeStruct.h:256).  They are instantiated
// with phi-free cones (PHI = false) for full polycones and with phi cones for sections;
// both are inline (a call would change the register allocation of the callers' loops).
__device__ __forceinline__ int pcon_n(const double *t) { return (int)t[row::PconNSec]; }
__device__ __forceinline__ const double *pcon_sec(const double *t, int n, int k) { return t + row::pcon_cone(n, k); }
__device__ __forceinline__ D3 pcon_local(const double *t, int n, int k, D3 p)
{
  return d3(p.x, p.y, p.z - t[row::pcon_shift(n) + k]);
}

// PolyconeStruct::GetSectionIndex (PolyconeStruct.h:302-311)
__device__ __forceinline__ int pcon_section_index(const double *t, int n, double zpos)
{
  const double *zs = t + row::PconZs;
  if (zpos < zs[0]) return -1;
  for (int i = 0; i < n; ++i)
    if (zpos >= zs[i] && zpos <= zs[i + 1]) return i;
  return -2;
}

// GenericKernelForASection (PolyconeImplementation.h:69-97)
template <bool PHI>
__device__ __forceinline__ void pcon_section_ci_t(const double *t, int n, int k, D3 p, bool forInside, bool &cin,
                                                bool &cout)
{
  if (k < 0) {
    cin  = false;
    cout = true;
    return;
  }
  cone_generic_ci<PHI>(pcon_sec(t, n, k), pcon_local(t, n, k, p), forInside, cin, cout);
}

// GenericKernelForContainsAndInside (PolyconeImplementation.h:127-187); cin/cout keep the
// caller's initial values where the reference leaves them untouched
template <bool PHI>
__device__ __forceinline__ void pcon_ci_t(const double *t, D3 p, bool forInside, bool &cin, bool &cout)
{
  const int n   = pcon_n(t);
  const int lo  = pcon_section_index(t, n, p.z - kTolerance);
  const int hi  = pcon_section_index(t, n, p.z + kTolerance);
  if (lo < 0 && hi < 0) {
    cout = true;
    return;
  }
  if (lo < 0 && hi == 0) {
    pcon_section_ci_t<PHI>(t, n, 0, p, forInside, cin, cout);
    return;
  }
  if (hi < 0 && lo == n - 1) {
    pcon_section_ci_t<PHI>(t, n, n - 1, p, forInside, cin, cout);
    return;
  }
  if (lo >= 0 && hi >= 0) {
    if (lo == hi) {
      pcon_section_ci_t<PHI>(t, n, lo, p, forInside, cin, cout);
      return;
    }
    bool inLo = false, outLo = false, inHi = false, outHi = false;
    pcon_section_ci_t<PHI>(t, n, lo, p, forInside, inLo, outLo);
    pcon_section_ci_t<PHI>(t, n, hi, p, forInside, inHi, outHi);
    if ((!inLo && !outLo) && (!inHi && !outHi)) {
      cin = true;
      return;
    }
    if (outLo && outHi) cout = true;
  }
}

template <bool PHI>
__device__ __forceinline__ bool pcon_contains_t(const double *t, D3 p)
{
  bool cin = false, cout = false;
  pcon_ci_t<PHI>(t, p, false, cin, cout);
  return !cout;
}

template <bool PHI>
__device__ __forceinline__ int pcon_inside_t(const double *t, D3 p)
{
  bool cin = false, cout = false;
  pcon_ci_t<PHI>(t, p, true, cin, cout);
  int r = kSurfaceE;
  if (cout) r = kOutsideE;
  if (cin) r = kInsideE;
  return r;
}

// DistanceToIn (PolyconeImplementation.h:189-237)
template <bool PHI>
__device__ __forceinline__ double pcon_dist_in_t(const double *t, D3 p, D3 v)
{
  const int n     = pcon_n(t);
  double distance = kInfLength;
  int increment   = (v.z > 0) ? 1 : -1;
  if (fabs(v.z) < kTolerance) increment = 0;
  int index = pcon_section_index(t, n, p.z);
  if (index == -1) index = 0;
  if (index == -2) index = n - 1;
  do {
    distance = cone_dist_in<PHI>(pcon_sec(t, n, index), pcon_local(t, n, index, p), v);
    if (distance < kInfLength || !increment) break;
    index += increment;
  } while (index >= 0 && index < n);
  return distance;
}

// DistanceToOut (PolyconeImplementation.h:239-379)
template <bool PHI>
__device__ __forceinline__ double pcon_dist_out_t(const double *t, D3 point, D3 dir)
{
  const int n = pcon_n(t);
  if (n == 1) return cone_dist_out<PHI>(pcon_sec(t, n, 0), pcon_local(t, n, 0, point), dir);
  const int lo = pcon_section_index(t, n, point.z - kTolerance);
  const int hi = pcon_section_index(t, n, point.z + kTolerance);
  int index    = 0;
  if (lo < 0 && hi < 0) {
    return -1;
  } else if (lo < 0 && hi >= 0) {
    index = hi;
    if (cone_inside<PHI>(pcon_sec(t, n, index), pcon_local(t, n, index, point)) == kOutsideE) return -1;
  } else if (lo != hi && lo >= 0) {
    index = cone_inside<PHI>(pcon_sec(t, n, lo), pcon_local(t, n, lo, point)) == kOutsideE ? hi : lo;
  } else {
    index = lo;
    if (index < 0) index = pcon_section_index(t, n, point.z);
  }
  if (index < 0) return 0.;
  if (cone_inside<PHI>(pcon_sec(t, n, index), pcon_local(t, n, index, point)) == kOutsideE) return -1;
  double totalDistance = 0.;
  int increment        = (dir.z > 0) ? 1 : -1;
  if (fabs(dir.z) < kTolerance) increment = 0;
  int istep = 0;
  D3 pn     = point;
  do {
    const double shift = t[row::pcon_shift(n) + index];
    if ((totalDistance != 0) || (istep < 2)) {
      pn = d3(point.x + totalDistance * dir.x, point.y + totalDistance * dir.y, point.z + totalDistance * dir.z);
      pn.z -= shift;
      if (cone_inside<PHI>(pcon_sec(t, n, index), pn) == kOutsideE) break;
    } else {
      pn.z -= shift;
    }
    istep++;
    const double dist = cone_dist_out<PHI>(pcon_sec(t, n, index), pn, dir);
    if (dist == -1) return kInfLength;
    if (fabs(dist) < 0.5 * kTolerance) {
      int index1 = index;
      if ((index > 0) && (index < n - 1)) {
        index1 += increment;
      } else {
        if ((index == 0) && (increment > 0)) index1 += increment;
        if ((index == n - 1) && (increment < 0)) index1 += increment;
      }
      const double td = totalDistance + dist;
      D3 pte          = d3(point.x + td * dir.x, point.y + td * dir.y, point.z + td * dir.z);
      pte.z -= t[row::pcon_shift(n) + index1];
      if (cone_inside<PHI>(pcon_sec(t, n, index1), pte) == kOutsideE || (increment == 0)) break;
    }
    totalDistance += dist;
    index += increment;
  } while (increment != 0 && index >= 0 && index < n);
  return totalDistance;
}

// neighbour scan shared by SafetyToIn and SafetyToOut (PolyconeImplementation.h:413-446, 487-513)
template <bool PHI>
__device__ __forceinline__ double pcon_scan_neighbours_t(const double *t, int n, int index, D3 p, double minSafety)
{
  const double *zs = t + row::PconZs;
  double zbase     = zs[index + 1];
  for (int i = index + 1; i < n; ++i) {
    if (zs[i] - zbase >= minSafety) break;
    const double s = cone_safe_in<PHI>(pcon_sec(t, n, i), pcon_local(t, n, i, p));
    if (s < minSafety) minSafety = s;
  }
  if (index > 0) {
    zbase = zs[index - 1];
    for (int i = index - 1; i >= 0; --i) {
      if (zbase - zs[i] >= minSafety) break;
      const double s = cone_safe_in<PHI>(pcon_sec(t, n, i), pcon_local(t, n, i, p));
      if (s < minSafety) minSafety = s;
    }
  }
  return minSafety;
}

// SafetyToIn (PolyconeImplementation.h:381-450)
template <bool PHI>
__device__ __forceinline__ double pcon_safe_in_t(const double *t, D3 p)
{
  const int n = pcon_n(t);
  int index   = pcon_section_index(t, n, p.z);
  bool needZ  = false;
  if (index < 0) {
    needZ = true;
    if (index == -1) index = 0;
    if (index == -2) index = n - 1;
  }
  const double safety = cone_safe_in<PHI>(pcon_sec(t, n, index), pcon_local(t, n, index, p));
  if (needZ || safety < kTolerance) return safety;
  return pcon_scan_neighbours_t<PHI>(t, n, index, p, safety);
}

// SafetyToOut (PolyconeImplementation.h:452-517); neighbours probed with the cone's SafetyToIn
template <bool PHI>
__device__ __forceinline__ double pcon_safe_out_t(const double *t, D3 p)
{
  bool cin = false, cout = false;
  pcon_ci_t<PHI>(t, p, true, cin, cout);
  if (cout) return -1;
  const int n     = pcon_n(t);
  const int index = pcon_section_index(t, n, p.z);
  if (index < 0) return -1;
  const double minSafety = cone_safe_out<PHI>(pcon_sec(t, n, index), pcon_local(t, n, index, p));
  if (minSafety == kInfLength) return 0.;
  if (minSafety < kTolerance) return 0.;
  return pcon_scan_neighbours_t<PHI>(t, n, index, p, minSafety);
}

__device__ __forceinline__ bool pcon_has_phi(const double *t) { return cone_has_phi(pcon_sec(t, pcon_n(t), 0)); }

__device__ __forceinline__ bool pcon_contains(const double *t, D3 p)
{
  return pcon_has_phi(t) ? pcon_contains_t<true>(t, p) : pcon_contains_t<false>(t, p);
}
__device__ __forceinline__ int pcon_inside(const double *t, D3 p)
{
  return pcon_has_phi(t) ? pcon_inside_t<true>(t, p) : pcon_inside_t<false>(t, p);
}
__device__ __forceinline__ double pcon_dist_in(const double *t, D3 p, D3 v)
{
  return pcon_has_phi(t) ? pcon_dist_in_t<true>(t, p, v) : pcon_dist_in_t<false>(t, p, v);
}
__device__ __forceinline__ double pcon_dist_out(const double *t, D3 p, D3 v)
{
  return pcon_has_phi(t) ? pcon_dist_out_t<true>(t, p, v) : pcon_dist_out_t<false>(t, p, v);
}
__device__ __forceinline__ double pcon_safe_in(const double *t, D3 p)
{
  return pcon_has_phi(t) ? pcon_safe_in_t<true>(t, p) : pcon_safe_in_t<false>(t, p);
}
__device__ __forceinline__ double pcon_safe_out(const double *t, D3 p)
{
  return pcon_has_phi(t) ? pcon_safe_out_t<true>(t, p) : pcon_safe_out_t<false>(t, p);
}

// ---------------------------------------------------------------- Orb
// kernel/OrbImplementation.h:60-225; row = fR (OrbStruct.h:19)
__device__ __forceinline__ double orb_mag2(D3 p) { return p.x * p.x + p.y * p.y + p.z * p.z; }

__device__ __forceinline__ bool orb_contains(const double *o, D3 p)  // GenericKernelForContainsAndInside
{
  const double rad2 = orb_mag2(p);
  const double tolR = o[0] + kTolerance;
  return !(rad2 >= tolR * tolR);
}

__device__ __forceinline__ int orb_inside(const double *o, D3 p)
{
  const double rad2 = orb_mag2(p);
  double tolR       = o[0] - kTolerance;
  const bool cin    = rad2 <= tolR * tolR;
  tolR              = o[0] + kTolerance;
  const bool cout   = rad2 >= tolR * tolR;
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

// DetectIntersectionAndCalculateDistance (OrbImplementation.h:197-220)
__device__ __forceinline__ bool orb_intersect(const double *o, D3 p, D3 d, bool toIn, double &dist)
{
  const double rad2    = orb_mag2(p);
  const double pDotV3D = p.x * d.x + p.y * d.y + p.z * d.z;
  const double c       = rad2 - o[0] * o[0];
  const double d2      = pDotV3D * pDotV3D - c;
  if (toIn) {
    if (d2 >= 0. && pDotV3D <= 0.) {
      dist = -pDotV3D - sqrt(fabs(d2));
      return true;
    }
    return false;
  }
  if (d2 >= 0.) {
    dist = -pDotV3D + sqrt(fabs(d2));
    return true;
  }
  return false;
}

__device__ __forceinline__ double orb_dist_in(const double *o, D3 p, D3 d)
{
  const double rad = sqrt(orb_mag2(p));
  if (rad < o[0] - kTolerance) return -1.;
  const double pDotV3D = p.x * d.x + p.y * d.y + p.z * d.z;
  if (rad >= o[0] - kTolerance && rad <= o[0] + kTolerance && pDotV3D < 0.) return 0.;
  double dist = kInfLength;
  return orb_intersect(o, p, d, true, dist) ? dist : kInfLength;
}

__device__ __forceinline__ double orb_dist_out(const double *o, D3 p, D3 d)
{
  const double rad = sqrt(orb_mag2(p));
  if (rad > o[0] + kTolerance) return -1.;
  const double pDotV3D = p.x * d.x + p.y * d.y + p.z * d.z;
  if (rad >= o[0] - kTolerance && rad <= o[0] + kTolerance && pDotV3D > 0.) return 0.;
  double dist = kInfLength;
  return orb_intersect(o, p, d, false, dist) ? dist : kInfLength;
}

__device__ __forceinline__ double orb_safe_in(const double *o, D3 p)
{
  const double rad = sqrt(orb_mag2(p));
  double safety    = rad - o[0];
  if (rad < o[0] - kTolerance) return -1.;
  if (rad > o[0] - kTolerance && rad < o[0] + kTolerance) safety = 0.;
  return safety;
}

__device__ __forceinline__ double orb_safe_out(const double *o, D3 p)
{
  const double rad = sqrt(orb_mag2(p));
  double safety    = o[0] - rad;
  if (rad > o[0] + kTolerance) return -1.;
  if (rad > o[0] - kTolerance && rad < o[0] + kTolerance) safety = 0.;
  return safety;
}

// ---------------------------------------------------------------- CutTube
// kernel/CutTubeImplementation.h:101-279 over CutPlanes (CutPlanes.h:101-166) and Plane
// (Plane.h:102-191); row: the tube's row (infinite half-length), then row::CutTube*
__device__ __forceinline__ double ct_plane(const double *r, int k, D3 p)  // Plane::DistPlane
{
  const double *n = r + (k ? row::CutTubeN1 : row::CutTubeN0);
  return p.x * n[0] + p.y * n[1] + p.z * n[2] + r[k ? row::CutTubeD1 : row::CutTubeD0];
}
__device__ __forceinline__ double ct_ndir(const double *r, int k, D3 d)
{
  const double *n = r + (k ? row::CutTubeN1 : row::CutTubeN0);
  return d.x * n[0] + d.y * n[1] + d.z * n[2];
}
__device__ __forceinline__ double ct_plane_dist_in(const double *r, int k, D3 p, D3 d)  // Plane::DistanceToIn
{
  const double ndd = nonzero(ct_ndir(r, k, d)), saf = ct_plane(r, k, p);
  return (ndd < 0. && saf > -kTolerance) ? -saf / ndd : -kInfLength;
}
__device__ __forceinline__ double ct_plane_dist_out(const double *r, int k, D3 p, D3 d)  // Plane::DistanceToOut
{
  const double ndd = nonzero(ct_ndir(r, k, d)), saf = ct_plane(r, k, p);
  double distance  = kInfLength;
  if (saf > kTolerance) distance = -kInfLength;
  if (ndd > 0. && saf < kTolerance) distance = -saf / ndd;
  return distance;
}
__device__ __forceinline__ int ct_planes_inside(const double *r, D3 p)
{
  const double d0 = ct_plane(r, 0, p), d1 = ct_plane(r, 1, p);
  int inside      = (d0 < 0.0 && d1 < 0.0) ? kInsideE : kOutsideE;
  if (fabs(d0) < kTolerance || fabs(d1) < kTolerance) inside = kSurfaceE;
  return inside;
}
__device__ __forceinline__ double ct_planes_dist_in(const double *r, D3 p, D3 d)
{
  double d0 = ct_plane_dist_in(r, 0, p, d);
  if (ct_ndir(r, 0, d) > 0.) d0 = -kInfLength;
  double d1 = ct_plane_dist_in(r, 1, p, d);
  if (ct_ndir(r, 1, d) > 0.) d1 = -kInfLength;
  return vmax(d0, d1);
}
__device__ __forceinline__ double ct_planes_dist_out(const double *r, D3 p, D3 d)
{
  return vmin(ct_plane_dist_out(r, 0, p, d), ct_plane_dist_out(r, 1, p, d));
}

__device__ __forceinline__ bool cuttube_contains(const double *r, D3 p)
{
  if (!(ct_plane(r, 0, p) < 0. && ct_plane(r, 1, p) < 0.)) return false;
  return tube_contains(r, p);
}

__device__ __forceinline__ int cuttube_inside(const double *r, D3 p)
{
  const int incp = ct_planes_inside(r, p);
  if (incp == kOutsideE) return kOutsideE;
  int inside = tube_inside(r, p);
  if (incp == kOutsideE || (incp == kSurfaceE && inside != kOutsideE)) inside = incp;
  return inside;
}

__device__ __forceinline__ double cuttube_dist_in_kernel(const double *r, D3 p, D3 d, double stepmax)
{
  double distance = kInfLength;
  int incp        = ct_planes_inside(r, p);
  int instart     = tube_inside(r, p);
  if (incp == kOutsideE || (incp == kSurfaceE && instart != kOutsideE)) instart = incp;
  if (instart == kInsideE) distance = -1.;
  double dplanes         = ct_planes_dist_in(r, p, d);
  const double safplanes = vmax(ct_plane(r, 0, p), ct_plane(r, 1, p));
  const bool hitplanes   = fabs(dplanes) < stepmax && safplanes > -kTolerance;
  if (incp != kInsideE && !hitplanes) return distance;
  D3 prop = p;
  if (!hitplanes) dplanes = 0.;
  if (hitplanes) {
    prop = d3(prop.x + dplanes * d.x, prop.y + dplanes * d.y, prop.z + dplanes * d.z);
    incp = ct_planes_inside(r, prop);
  }
  bool done = incp == kOutsideE;
  done |= instart == kInsideE;
  if (done) return distance;
  instart           = tube_inside(r, prop);
  const bool inside = hitplanes && instart != kOutsideE;
  if (inside && !done) distance = dplanes;
  done |= inside;
  if (done) {
    if (fabs(distance) < kTolerance) distance = 0.;
    return distance;
  }
  const double dexit = ct_planes_dist_out(r, prop, d);
  double dtube       = tube_dist_in_kernel(r, prop, d);
  if (dtube < 0.) dtube = 0.;
  if (dexit < dtube) dtube = kInfLength;
  if (!done && (dtube + dplanes) < stepmax) distance = dtube + dplanes;
  return distance;
}

__device__ __forceinline__ double cuttube_dist_in(const double *r, D3 pt, D3 d, double stepmax)
{
  D3 p                = pt;
  const double ptDist = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double distToMove   = 0.;
  const double order  = 100.;
  if (ptDist > order * r[row::CutTubeMaxVal]) {
    distToMove = ptDist - order * r[row::CutTubeMaxVal];
    p          = d3(p.x + distToMove * d.x, p.y + distToMove * d.y, p.z + distToMove * d.z);
  }
  double distance = cuttube_dist_in_kernel(r, p, d, stepmax);
  distance += distToMove;
  return distance;
}

__device__ __forceinline__ double cuttube_dist_out(const double *r, D3 p, D3 d)
{
  double distance    = ct_planes_dist_out(r, p, d);
  const double dtube = tube_dist_out(r, p, d);
  if (dtube < distance) distance = dtube;
  return distance;
}

__device__ __forceinline__ double cuttube_safe_in(const double *r, D3 p)
{
  double safety        = vmax(ct_plane(r, 0, p), ct_plane(r, 1, p));
  const double saftube = tube_safe_in(r, p);
  if (saftube > safety) safety = saftube;
  return safety;
}

__device__ __forceinline__ double cuttube_safe_out(const double *r, D3 p)
{
  double safety        = vmin(-ct_plane(r, 0, p), -ct_plane(r, 1, p));
  const double saftube = tube_safe_out(r, p);
  if (saftube < safety) safety = saftube;
  return safety;
}

// ---------------------------------------------------------------- Polyhedron
// PolyhedronImplementation.h over a row::Phd* row (Quadrilaterals.h, Planes.h for the faces).
// The reference's placement specialisation by inner radii and phi cut-out
// (UnplacedPolyhedron.cpp:75-103) behaves as the generic kernel with the shape's own flags.
// The six entry points are out of line: they loop over faces and would otherwise be inlined
// into every kernel that dispatches on the shape type.  Compiled in the sections kernel set
// only (a geometry holding a polyhedron runs that set): the calls' register saves would
// otherwise cost the full-range kernels spills.
#if VGN_SECTIONS
namespace ph = row;

struct PhdSeg {
  const double *outer, *phi, *inner;
  int no, np, ni;
};

__device__ __forceinline__ PhdSeg phd_seg(const double *r, int si)
{
  const int nz = (int)r[ph::PhdNz], S = (int)r[ph::PhdSides];
  const double *st = r + ph::phd_segs(nz, S) + 4 * si;
  PhdSeg s;
  s.no    = (int)st[0];
  s.np    = (int)st[1];
  s.ni    = (int)st[2];
  s.outer = r + (int64_t)st[3];
  s.phi   = s.outer + s.no * ph::kQuadSize;
  s.inner = s.phi + s.np * ph::kQuadSize;
  return s;
}

__device__ __forceinline__ bool phd_has_phi(const double *r) { return r[ph::PhdHasPhi] != 0.; }
__device__ __forceinline__ D3 quad_n(const double *q) { return d3(q[ph::QuadN], q[ph::QuadN + 1], q[ph::QuadN + 2]); }
__device__ __forceinline__ D3 quad_side(const double *q, int j)
{
  return d3(q[ph::QuadSide + 4 * j], q[ph::QuadSide + 4 * j + 1], q[ph::QuadSide + 4 * j + 2]);
}
__device__ __forceinline__ D3 quad_corner(const double *q, int j)
{
  return d3(q[ph::QuadCorner + 3 * j], q[ph::QuadCorner + 3 * j + 1], q[ph::QuadCorner + 3 * j + 2]);
}

// Quadrilaterals::RayHitsQuadrilateral (Quadrilaterals.h:139-150)
__device__ __forceinline__ bool quad_ray_hits(const double *q, D3 x)
{
  for (int j = 0; j < 4; ++j)
    if (!(dot3(x, quad_side(q, j)) + q[ph::QuadSide + 4 * j + 3] >= -kTolerance)) return false;
  return true;
}

// Quadrilaterals::DistanceToIn<double, behindPlanesT> (Quadrilaterals.h:361-396)
template <bool BEHIND>
__device__ __forceinline__ double quads_dist_in(const double *q, int n, D3 p, D3 d)
{
  double best = kInfLength;
  for (int i = 0; i < n; ++i, q += ph::kQuadSize) {
    const D3 nn = quad_n(q);
    double dist = dot3(p, nn) + q[ph::QuadD];
    if (!((BEHIND ? -dist : dist) > -kTolerance)) continue;
    const double proj = dot3(d, nn);
    if (!((BEHIND ? proj : -proj) > 0)) continue;
    dist /= -(proj + copysign(1E-20, proj));
    if (quad_ray_hits(q, d3(p.x + dist * d.x, p.y + dist * d.y, p.z + dist * d.z))) best = dist;
    if (best < kInfLength) break;
  }
  return 0. > best ? 0. : best;
}

// Quadrilaterals::DistanceToOut(point, direction, zMin, zMax) (Quadrilaterals.h:466-516)
__device__ __forceinline__ double quads_dist_out(const double *q, int n, D3 p, D3 d, double zMin, double zMax)
{
  double best = kInfLength;
  for (int i = 0; i < n; ++i, q += ph::kQuadSize) {
    const D3 nn = quad_n(q);
    double dt   = dot3(p, nn) + q[ph::QuadD];
    if (!(dt < kTolerance)) continue;
    const double proj = dot3(d, nn);
    if (!(proj > 0)) continue;
    dt /= -proj;
    if (!(dt < best)) continue;
    bool valid;
    if (zMin == zMax) {
      valid = quad_ray_hits(q, d3(p.x + dt * d.x, p.y + dt * d.y, p.z + dt * d.z));
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

__device__ __forceinline__ double mag2_3(D3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

// DistanceToLineSegmentSquared1 (GenericKernels.h:188-215)
__device__ __forceinline__ double phd_segment_dist2(D3 c0, D3 c1, D3 p)
{
  double result = kInfLength;
  const D3 line = d3(c1.x - c0.x, c1.y - c0.y, c1.z - c0.z);
  const D3 pc0  = d3(p.x - c0.x, p.y - c0.y, p.z - c0.z);
  const double dot0 = dot3(pc0, line);
  if (dot0 <= 0) return mag2_3(pc0);
  const double dot1 = mag2_3(line);
  if (dot1 <= dot0) result = mag2_3(d3(p.x - c1.x, p.y - c1.y, p.z - c1.z));
  if (result < kInfLength) return result;
  const double f = dot0 / dot1;
  return mag2_3(d3((c0.x + f * line.x) - p.x, (c0.y + f * line.y) - p.y, (c0.z + f * line.z) - p.z));
}

// Quadrilaterals::ScalarDistanceSquared (Quadrilaterals.h:535-572)
__device__ __forceinline__ double quad_dist2(const double *q, D3 p)
{
  const D3 n      = quad_n(q);
  double distance = dot3(p, n) + q[ph::QuadD];
  const D3 x      = d3(p.x - distance * n.x, p.y - distance * n.y, p.z - distance * n.z);
  bool within[4];
  for (int j = 0; j < 4; ++j) {
    const double *s = q + ph::QuadSide + 4 * j;
    within[j]       = x.x * s[0] + x.y * s[1] + x.z * s[2] + s[3] >= 0;
  }
  if (within[0] && within[1] && within[2] && within[3]) return distance * distance;
  double dsq = kInfLength;
  for (int j = 0; j < 4; ++j) {
    if (!within[j]) {
      distance = phd_segment_dist2(quad_corner(q, j), quad_corner(q, (j + 1) % 4), p);
      if (distance < dsq) dsq = distance;
    }
  }
  return dsq;
}

// Planes::Contains (Planes.h:192-205)
__device__ __forceinline__ bool quads_contains(const double *q, int n, D3 p)
{
  bool r = true;
  for (int i = 0; i < n; ++i, q += ph::kQuadSize) r &= dot3(p, quad_n(q)) + q[ph::QuadD] < 0;
  return r;
}

// Planes::Inside of one plane (Planes.h:268-281)
__device__ __forceinline__ int quad_inside(const double *q, D3 p)
{
  const double dist = q[0] * p.x + q[1] * p.y + q[2] * p.z + q[ph::QuadD];
  if (dist > kHalfTolerance) return kOutsideE;
  if (dist > -kHalfTolerance) return kSurfaceE;
  return kInsideE;
}

// Planes::Inside over all planes (Planes.h:246-266)
__device__ __forceinline__ int quads_inside(const double *q, int n, D3 p)
{
  int r = kInsideE;
  for (int i = 0; i < n; ++i, q += ph::kQuadSize) {
    const double dist = q[0] * p.x + q[1] * p.y + q[2] * p.z + q[ph::QuadD];
    if (dist > kHalfTolerance) r = kOutsideE;
    if (r == kInsideE && dist > -kHalfTolerance) r = kSurfaceE;
    if (r == kOutsideE) break;
  }
  return r;
}

// FindZSegmentKernel<double> (PolyhedronImplementation.h:232-244)
__device__ __forceinline__ int phd_find_z(const double *r, double pz)
{
  const int nz    = (int)r[ph::PhdNz];
  const double *z = r + ph::phd_z(nz);
  int index = -1, b = 0;
  while (b < nz - 1 && pz - kTolerance > z[b]) {
    ++index;
    ++b;
  }
  if (pz + kTolerance > z[b]) return index + 1;
  return index;
}

// FindPhiSegment (PolyhedronImplementation.h:256-276)
__device__ __forceinline__ int phd_find_phi(const double *r, D3 p)
{
  const int nz = (int)r[ph::PhdNz], S = (int)r[ph::PhdSides];
  const double *s = r + ph::phd_phisec(nz);
  int index       = -1;
  double first    = p.x * s[0] + p.y * s[1] + p.z * s[2];
  for (int i = 1; i < S + 1; ++i) {
    const double second = p.x * s[3 * i] + p.y * s[3 * i + 1] + p.z * s[3 * i + 2];
    if (first > -kTolerance && second < kTolerance) index = i - 1;
    if (index >= 0) break;
    first = second;
  }
  return index;
}

__device__ __forceinline__ int phd_clamp_z(const double *r, int z)
{
  const int zmax = (int)r[ph::PhdNz] - 1;
  return z < 0 ? 0 : (z >= zmax ? zmax - 1 : z);
}

// DistanceToInZSegment (PolyhedronImplementation.h:278-318)
__device__ __forceinline__ double phd_dist_in_seg(const double *r, int si, D3 p, D3 d)
{
  const PhdSeg sg = phd_seg(r, si);
  double distance = quads_dist_in<false>(sg.outer, sg.no, p, d);
  if (distance < kInfLength) return distance;
  if (phd_has_phi(r)) distance = quads_dist_in<false>(sg.phi, sg.np, p, d);
  if (distance < kInfLength) return distance;
  if (sg.ni > 0) distance = quads_dist_in<true>(sg.inner, sg.ni, p, d);
  return distance;
}

// DistanceToOutZSegment (PolyhedronImplementation.h:320-362)
__device__ __forceinline__ double phd_dist_out_seg(const double *r, int si, double zMin, double zMax, D3 p, D3 d)
{
  const PhdSeg sg = phd_seg(r, si);
  bool done       = false;
  double distance = kInfLength;
  if (sg.ni > 0) {
    distance = quads_dist_in<false>(sg.inner, sg.ni, p, d);
    done     = distance < kInfLength;
    if (done) return distance;
  }
  if (phd_has_phi(r)) {
    const double distphi = quads_dist_in<true>(sg.phi, sg.np, p, d);
    if (!done && distance > -kTolerance) distance = distphi;
    done = distance > -kTolerance && distance < kInfLength;
    if (done) return distance;
  }
  const double distout = quads_dist_out(sg.outer, sg.no, p, d, zMin, zMax);
  if (!done) distance = distout;
  return distance;
}

// InPhiCutoutWedge (PolyhedronImplementation.h:541-555)
__device__ __forceinline__ bool phd_in_cutout(const PhdSeg &sg, bool large, D3 p)
{
  const bool s0 = dot3(p, quad_n(sg.phi)) + sg.phi[ph::QuadD] >= 0;
  const bool s1 = dot3(p, quad_n(sg.phi + ph::kQuadSize)) + sg.phi[ph::kQuadSize + ph::QuadD] >= 0;
  return large ? (s0 || s1) : (s0 && s1);
}

// ScalarSafetyToZSegmentSquared (PolyhedronImplementation.h:364-466); `phiIndex` may move to
// the first or last side, as in the reference
__device__ __forceinline__ double phd_safety_seg2(const double *r, int si, int &phiIndex, D3 p, bool pt_inside)
{
  const PhdSeg sg      = phd_seg(r, si);
  const int nz         = (int)r[ph::PhdNz];
  const bool in_cutout = phiIndex < 0;
  double s2            = kInfLength;
  if (phd_has_phi(r) && sg.np == 2) {
    if (pt_inside || in_cutout) {
      s2               = quad_dist2(sg.phi, p);
      const double saf = quad_dist2(sg.phi + ph::kQuadSize, p);
      if (saf < s2) s2 = saf;
      if (in_cutout) {
        if (r[ph::PhdLargePhi] != 0. && sg.ni > 0) {
          double si2 = quad_dist2(sg.inner, p);
          if (si2 < s2) {
            phiIndex = 0;
            s2       = si2;
          }
          if (sg.ni > 1) {
            si2 = quad_dist2(sg.inner + (sg.ni - 1) * ph::kQuadSize, p);
            if (si2 < s2) {
              phiIndex = sg.ni - 1;
              s2       = si2;
            }
          }
        }
        return s2;
      }
    }
  }
  if (in_cutout && si > 0 && si < nz - 2 && r[ph::phd_z(nz) + si] == r[ph::phd_z(nz) + si + 1]) {
    if (sg.no > 0) {
      double so = quad_dist2(sg.outer, p);
      if (so < s2) {
        phiIndex = 0;
        s2       = so;
      }
      if (sg.no > 1) {
        so = quad_dist2(sg.outer + (sg.no - 1) * ph::kQuadSize, p);
        if (so < s2) {
          phiIndex = sg.no - 1;
          s2       = so;
        }
      }
    }
    if (sg.ni > 0) {
      double si2 = quad_dist2(sg.inner, p);
      if (si2 < s2) {
        phiIndex = 0;
        s2       = si2;
      }
      if (sg.ni > 1) {
        si2 = quad_dist2(sg.inner + (sg.ni - 1) * ph::kQuadSize, p);
        if (si2 < s2) {
          phiIndex = sg.ni - 1;
          s2       = si2;
        }
      }
    }
    return s2;
  }
  const double so  = sg.no > 0 ? quad_dist2(sg.outer + phiIndex * ph::kQuadSize, p) : kInfLength;
  const double si2 = sg.ni > 0 ? quad_dist2(sg.inner + phiIndex * ph::kQuadSize, p) : kInfLength;
  if (si2 < s2) s2 = si2;
  if (so < s2) s2 = so;
  return s2;
}

// ScalarDistanceToEndcaps<pointInsideT> (PolyhedronImplementation.h:468-511)
template <bool INSIDE>
__device__ __forceinline__ void phd_dist_endcaps(const double *r, D3 p, D3 d, double &distance)
{
  const int nz = (int)r[ph::PhdNz], nseg = nz - 1;
  const bool last     = INSIDE ? !(d.z < 0) : (d.z < 0);
  const PhdSeg sg     = phd_seg(r, last ? nseg - 1 : 0);
  const double zPlane = r[ph::phd_z(nz) + (last ? nseg : 0)];
  const double dt     = (zPlane - p.z) / nonzero(d.z);
  if (dt < -kTolerance || dt >= distance) return;
  const D3 x = d3(p.x + dt * d.x, p.y + dt * d.y, p.z + dt * d.z);
  if (!quads_contains(sg.outer, sg.no, x)) return;
  if (sg.ni > 0 && quads_contains(sg.inner, sg.ni, x)) return;
  if (phd_has_phi(r) && phd_in_cutout(sg, r[ph::PhdLargePhi] != 0., x)) return;
  distance = dt;
}

// ScalarSafetyToEndcapsSquared (PolyhedronImplementation.h:513-539)
__device__ __forceinline__ void phd_safety_endcaps2(const double *r, D3 p, double &dist2)
{
  const int nz = (int)r[ph::PhdNz], nseg = nz - 1;
  const double first  = r[ph::phd_z(nz)] - p.z;
  const double lastd  = r[ph::phd_z(nz) + nseg] - p.z;
  const bool isFirst  = fabs(first) < fabs(lastd);
  const PhdSeg sg     = phd_seg(r, isFirst ? 0 : nseg - 1);
  const double dt     = isFirst ? first : lastd;
  const double dt2    = dt * dt;
  if (dt2 >= dist2) return;
  const D3 x = d3(p.x, p.y, p.z + dt);
  if (!quads_contains(sg.outer, sg.no, x)) return;
  if (sg.ni > 0 && quads_contains(sg.inner, sg.ni, x)) return;
  if (phd_has_phi(r) && phd_in_cutout(sg, r[ph::PhdLargePhi] != 0., x)) return;
  dist2 = dt2;
}

// Wedge::Inside (Wedge_Evolution.h:262-272)
__device__ __forceinline__ int phd_wedge_inside(const double *w, D3 p)
{
  bool cin = false, cout = false;
  wedge_ci<true>(w, p, cin, cout);
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

// ScalarInsideSegBorder (PolyhedronImplementation.h:628-664)
__device__ __forceinline__ int phd_inside_border(const double *r, D3 p, int zi)
{
  const int nz = (int)r[ph::PhdNz];
  const PhdSeg sg    = phd_seg(r, zi);
  const int phiIndex = phd_find_phi(r, p);
  if (phiIndex < 0) return kOutsideE;
  const double *q  = (sg.no ? sg.outer : sg.inner) + phiIndex * ph::kQuadSize;
  const double rr  = fabs(dot3(p, quad_side(q, 0)));
  const double *rn = r + ph::phd_rmin(nz), *rx = r + ph::phd_rmax(nz);
  const bool in1   = (rr > rn[zi] - kTolerance) && (rr < rx[zi] + kTolerance);
  const bool in2   = (rr > rn[zi + 1] - kTolerance) && (rr < rx[zi + 1] + kTolerance);
  if (in1 && in2) {
    if ((rr < rn[zi] + kTolerance) || (rr > rx[zi] - kTolerance) || (rr < rn[zi + 1] + kTolerance) ||
        (rr > rx[zi + 1] - kTolerance))
      return kSurfaceE;
    if (phd_has_phi(r)) return phd_wedge_inside(r + ph::PhdWedge, p);
    return kInsideE;
  }
  if (!in1 && !in2) return kOutsideE;
  return kSurfaceE;
}

// ScalarInsideSegPhi (PolyhedronImplementation.h:666-701)
__device__ __forceinline__ int phd_inside_seg_phi(const double *r, D3 p, int zi, int phiIndex)
{
  if (phiIndex < 0) return kOutsideE;
  const int nz    = (int)r[ph::PhdNz];
  const double dz = fabs(p.z - r[ph::PhdTubeOffset]) - 0.5 * (r[ph::phd_z(nz) + nz - 1] - r[ph::phd_z(nz)]);
  if (dz > kHalfTolerance) return kOutsideE;
  if (r[ph::phd_samez(nz) + zi] != 0.) return phd_inside_border(r, p, zi);
  const PhdSeg sg = phd_seg(r, zi);
  int res         = quad_inside(sg.outer + phiIndex * ph::kQuadSize, p);
  if (res != kInsideE) return res;
  if (sg.ni > 0) {
    res = quad_inside(sg.inner + phiIndex * ph::kQuadSize, p);
    if (res == kInsideE) return kOutsideE;
    if (res == kSurfaceE) return kSurfaceE;
  }
  if (phd_has_phi(r)) {
    res = phd_wedge_inside(r + ph::PhdWedge, p);
    if (res != kInsideE) return res;
  }
  if (fabs(dz) < kHalfTolerance) return kSurfaceE;
  return kInsideE;
}

// ScalarContainsKernel (PolyhedronImplementation.h:557-592)
__device__ __noinline__ bool polyhedron_contains(const double *r, D3 p)
{
  if (!tube_contains(r + ph::PhdTube, d3(p.x, p.y, p.z - r[ph::PhdTubeOffset]))) return false;
  const int nz = (int)r[ph::PhdNz];
  const int zi = phd_find_z(r, p.z);
  if (!(zi >= 0 && zi < nz - 1)) return false;
  const PhdSeg sg = phd_seg(r, zi);
  if (r[ph::phd_samez(nz) + zi] != 0.) {
    const int phiIndex = phd_find_phi(r, p);
    if (phiIndex < 0) return false;
    const double *q  = (sg.no ? sg.outer : sg.inner) + phiIndex * ph::kQuadSize;
    const double rr  = fabs(dot3(p, quad_side(q, 0)));
    const double *rn = r + ph::phd_rmin(nz), *rx = r + ph::phd_rmax(nz);
    return ((rr >= rn[zi]) && (rr <= rx[zi])) | ((rr >= rn[zi + 1]) && (rr <= rx[zi + 1]));
  }
  if (!quads_contains(sg.outer, sg.no, p)) return false;
  if (sg.ni > 0 && quads_contains(sg.inner, sg.ni, p)) return false;
  if (phd_has_phi(r) && !quads_contains(sg.phi, sg.np, p)) return false;
  return true;
}

// ScalarInsideKernel (PolyhedronImplementation.h:594-626)
__device__ __forceinline__ int polyhedron_inside_kernel(const double *r, D3 p)
{
  if (!tube_contains(r + ph::PhdTube, d3(p.x, p.y, p.z - r[ph::PhdTubeOffset]))) return kOutsideE;
  const int nz = (int)r[ph::PhdNz];
  int zi       = phd_find_z(r, p.z);
  if (zi > nz - 2) zi = nz - 2;
  if (zi < 0) zi = 0;
  if (r[ph::phd_samez(nz) + zi] != 0.) return phd_inside_border(r, p, zi);
  const PhdSeg sg = phd_seg(r, zi);
  int res         = quads_inside(sg.outer, sg.no, p);
  if (res != kInsideE) return res;
  if (sg.ni > 0) {
    res = quads_inside(sg.inner, sg.ni, p);
    if (res == kInsideE) return kOutsideE;
    if (res == kSurfaceE) return kSurfaceE;
  }
  if (phd_has_phi(r)) {
    res = quads_inside(sg.phi, sg.np, p);
    if (res != kInsideE) return res;
  }
  const double dz =
      fabs(fabs(p.z - r[ph::PhdTubeOffset]) - 0.5 * (r[ph::phd_z(nz) + nz - 1] - r[ph::phd_z(nz)]));
  if (dz < kTolerance) return kSurfaceE;
  return kInsideE;
}

__device__ __noinline__ int polyhedron_inside(const double *r, D3 p) { return polyhedron_inside_kernel(r, p); }

// ScalarDistanceToInKernel (PolyhedronImplementation.h:703-751)
__device__ __noinline__ double polyhedron_dist_in(const double *r, D3 p, D3 d)
{
  const int nz = (int)r[ph::PhdNz], nseg = nz - 1;
  const double *z = r + ph::phd_z(nz);
  if ((p.z < z[0] + kTolerance) && d.z <= 0) return kInfLength;
  if ((p.z > z[nseg] - kTolerance) && d.z >= 0) return kInfLength;
  if (polyhedron_inside_kernel(r, p) == kInsideE) return -1.;
  double tubeDistance = 0., distance = kInfLength;
  const D3 bp = d3(p.x, p.y, p.z - r[ph::PhdTubeOffset]);
  if (!tube_contains(r + ph::PhdTube, bp)) {
    tubeDistance = tube_dist_in(r + ph::PhdTube, bp, d);
    if (tubeDistance == kInfLength) return kInfLength;
  }
  int zi = phd_clamp_z(r, phd_find_z(r, p.z));
  if (d.z >= 0) {
    for (; zi < nseg; ++zi) {
      distance = phd_dist_in_seg(r, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = phd_dist_in_seg(r, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  }
  phd_dist_endcaps<false>(r, p, d, distance);
  return (distance >= tubeDistance - 1E-6) ? distance : kInfLength;
}

// ScalarDistanceToOutKernel (PolyhedronImplementation.h:868-914)
__device__ __noinline__ double polyhedron_dist_out(const double *r, D3 p, D3 d)
{
  const int nz = (int)r[ph::PhdNz], nseg = nz - 1;
  const double *z = r + ph::phd_z(nz);
  if ((p.z < z[0] - kTolerance) || (p.z > z[nseg] + kTolerance)) return -1.;
  if (polyhedron_inside_kernel(r, p) == kOutsideE) return -1.;
  double distance = kInfLength;
  int zi          = phd_clamp_z(r, phd_find_z(r, p.z));
  if (d.z >= 0) {
    for (; zi < nseg; ++zi) {
      distance = phd_dist_out_seg(r, zi, z[zi], z[zi + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (z[zi] - p.z > distance) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = phd_dist_out_seg(r, zi, z[zi], z[zi + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (p.z - z[zi] > distance) break;
    }
  }
  phd_dist_endcaps<true>(r, p, d, distance);
  if (distance >= kInfLength) distance = 0.;
  return distance;
}

// ScalarSafetyKernel (PolyhedronImplementation.h:753-800)
__device__ __noinline__ double polyhedron_safety(const double *r, D3 p, bool pt_inside)
{
  const int nz = (int)r[ph::PhdNz], nseg = nz - 1;
  const double *z = r + ph::phd_z(nz);
  double safety   = kInfLength;
  const int zi    = phd_clamp_z(r, phd_find_z(r, p.z));
  int phiIndex    = phd_find_phi(r, p);
  const int in    = phd_inside_seg_phi(r, p, zi, phiIndex);
  if (in == kSurfaceE) return 0.;
  if ((in == kInsideE) ^ pt_inside) return -1.;
  for (int k = zi; k < nseg;) {
    const double s = phd_safety_seg2(r, k, phiIndex, p, pt_inside);
    safety         = safety < s ? safety : s;
    ++k;
    const double dz = z[k] - p.z;
    if (dz * dz > safety) break;
  }
  for (int k = zi - 1; k >= 0; --k) {
    const double s = phd_safety_seg2(r, k, phiIndex, p, pt_inside);
    safety         = safety < s ? safety : s;
    const double dz = p.z - z[k];
    if (dz * dz > safety) break;
  }
  phd_safety_endcaps2(r, p, safety);
  return sqrt(safety);
}
#endif  // VGN_SECTIONS

// ---------------------------------------------------------------- Torus2
// kernel/TorusImplementation2.h over a row::Tor* row.  Compiled in the sections kernel set only
// (a geometry holding a torus runs that set); the six entry points are out of line, as the
// polyhedron's are.  The cubic solver's cbrt, pow, cos and atan2 are written out with IEEE
// operations only (+, -, *, /, sqrt), identically in the oracle, so the two agree bit for bit;
// the reference calls the C library's, which these match to a few units in the last place.
#if VGN_SECTIONS
namespace tr = row;

// cube root of a >= 0: a = m 2^(3q), m in [0.5, 4); Newton's iteration from a linear start
__device__ __forceinline__ double tor_cbrt(double a)
{
  if (a == 0.0 || !(a < kInfLength)) return a;
  int e;
  double m = frexp(a, &e);
  int r    = e % 3;
  if (r < 0) r += 3;
  m = ldexp(m, r);
  e -= r;
  double y = 0.6 + 0.25 * m;
  for (int k = 0; k < 6; ++k) y = (2.0 * y + m / (y * y)) / 3.0;
  return ldexp(y, e / 3);
}

__device__ __forceinline__ double tor_pow16(double a) { return sqrt(tor_cbrt(a)); }

// atan(z), 0 <= z <= 1: two argument halvings, then the Taylor series to z^23
__device__ __forceinline__ double tor_atan_unit(double z)
{
  z = z / (1.0 + sqrt(1.0 + z * z));
  z = z / (1.0 + sqrt(1.0 + z * z));
  const double z2 = z * z;
  double term = z, s = z;
  for (int k = 1; k < 12; ++k) {
    term *= -z2;
    s += term / (2 * k + 1);
  }
  return 4.0 * s;
}

__device__ __forceinline__ double tor_atan2(double y, double x)  // y > 0
{
  const double ax = fabs(x);
  const double a  = (y <= ax) ? tor_atan_unit(y / ax) : 0.5 * kPiD - tor_atan_unit(ax / y);
  return x < 0 ? kPiD - a : a;
}

__device__ __forceinline__ double tor_cos(double w)  // |w| <= 1.1
{
  const double w2 = w * w;
  double term = 1.0, s = 1.0;
  for (int k = 1; k <= 12; ++k) {
    term *= -w2 / ((2 * k - 1) * (2 * k));
    s += term;
  }
  return s;
}

// SolveCubic (TorusImplementation2.h:17-53)
__device__ __forceinline__ unsigned tor_solve_cubic(double a, double b, double c, double *x)
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

__device__ __forceinline__ void tor_cmp_swap(double *v, int i, int j)  // CmpAndSwap
{
  if (v[i] > v[j]) {
    const double c = v[j];
    v[j]           = v[i];
    v[i]           = c;
  }
}

__device__ __forceinline__ void tor_sort4(double *v)  // Sort4 (TorusImplementation2.h:68-77)
{
  tor_cmp_swap(v, 0, 2);
  tor_cmp_swap(v, 1, 3);
  tor_cmp_swap(v, 0, 1);
  tor_cmp_swap(v, 2, 3);
  tor_cmp_swap(v, 1, 2);
}

// SolveQuartic (TorusImplementation2.h:79-150)
__device__ __forceinline__ int tor_solve_quartic(double a, double b, double c, double d, double *x)
{
  const double e = b - 3. * a * a / 8.;
  const double f = c + a * a * a / 8. - 0.5 * a * b;
  const double g = d - 3. * a * a * a * a / 256. + a * a * b / 16. - a * c / 4.;
  double xx[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  double delta, h = 0.;
  unsigned ireal = 0;
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
    x[ireal++]            = -0.25 * a;
    const unsigned ncubic = tor_solve_cubic(0, e, f, xx);
    for (unsigned i = 0; i < ncubic; i++) x[ireal++] = xx[i] - 0.25 * a;
    tor_sort4(x);
    return (int)ireal;
  }
  ireal = tor_solve_cubic(2. * e, e * e - 4. * g, -f * f, xx);
  if (ireal == 1) {
    if (xx[0] <= 0) return 0;
    h = sqrt(xx[0]);
  } else {
    for (unsigned i = 0; i < 3; i++) {
      h = xx[i];
      if (h >= 0) break;
    }
    if (h <= 0) return 0;
    h = sqrt(h);
  }
  const double j = 0.5 * (e + h * h - f / h);
  ireal          = 0;
  delta          = h * h - 4. * j;
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

__device__ __forceinline__ bool torus_has_phi(const double *t) { return t[tr::TorDphi] < 2. * kPiD; }

// GenericKernelForContainsAndInside<ForInside, notForDisk> (TorusImplementation2.h:241-285)
template <bool FOR_INSIDE, bool NOT_FOR_DISK>
__device__ __forceinline__ void torus_ci(const double *t, D3 p, bool &cin, bool &cout)
{
  const double tol   = 100. * kTolerance;
  const double rtor  = t[tr::TorRtor];
  const double rxy   = sqrt(p.x * p.x + p.y * p.y);
  const double radsq = (rxy - rtor) * (rxy - rtor) + p.z * p.z;
  if (FOR_INSIDE) {
    cout = radsq > (tol * t[tr::TorRmax] + t[tr::TorRmax2]);
    cin  = radsq < (-tol * t[tr::TorRmax] + t[tr::TorRmax2]);
  } else {
    cout = radsq > t[tr::TorRmax2];
  }
  if (cout) return;
  if (FOR_INSIDE) {
    cout |= radsq < (-tol * t[tr::TorRmin] + t[tr::TorRmin2]);
    cin &= radsq > (tol * t[tr::TorRmin] + t[tr::TorRmin2]);
  } else {
    cout |= radsq < t[tr::TorRmin2];
  }
  if (cout) return;
  if (NOT_FOR_DISK && torus_has_phi(t)) {
    bool cinphi = false, coutphi = false;
    wedge_ci<FOR_INSIDE>(t + tr::TorWedge, p, cinphi, coutphi);
    cout |= coutphi;
    if (FOR_INSIDE) cin &= cinphi;
  }
}

__device__ __forceinline__ int torus_inside_kernel(const double *t, D3 p)  // InsideKernel
{
  bool cin = false, cout = false;
  torus_ci<true, true>(t, p, cin, cout);
  return cout ? kOutsideE : (cin ? kInsideE : kSurfaceE);
}

__device__ __forceinline__ bool torus_contains_disk(const double *t, D3 p)  // UnplacedContainsDisk
{
  bool cin = false, cout = false;
  torus_ci<false, false>(t, p, cin, cout);
  return !cout;
}

// ToBoundary<ForRmin> (TorusImplementation2.h:287-377)
__device__ __forceinline__ double torus_to_boundary(const double *t, D3 pt, D3 dir, double radius, bool out)
{
  const double tol    = 100. * kTolerance;
  const double rtor = t[tr::TorRtor], rtor2 = t[tr::TorRtor2];
  const double r0sq   = pt.x * pt.x + pt.y * pt.y + pt.z * pt.z;
  const double rdotn  = pt.x * dir.x + pt.y * dir.y + pt.z * dir.z;
  const double rsumsq = rtor2 + radius * radius;
  const double a      = 4. * rdotn;
  const double b      = 2. * (r0sq + 2. * rdotn * rdotn - rsumsq + 2. * rtor2 * dir.z * dir.z);
  const double c      = 4. * (r0sq * rdotn - rsumsq * rdotn + 2. * rtor2 * pt.z * dir.z);
  const double d      = r0sq * r0sq - 2. * r0sq * rsumsq + 4. * rtor2 * pt.z * pt.z +
                   (rtor2 - radius * radius) * (rtor2 - radius * radius);
  double x[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  int nsol    = 0;
  if (fabs(dir.z) < 1E-3 && fabs(pt.z) < 0.1 * radius) {
    double r0            = rtor - sqrt((radius - pt.z) * (radius + pt.z));
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
    r0    = rtor + sqrt((radius - pt.z) * (radius + pt.z));
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
  const bool inner = fabs(radius - t[tr::TorRmin]) < kTolerance;
  for (int i = 0; i < nsol; i++) {
    if (x[i] < -10) continue;
    D3 r0         = d3(pt.x + x[i] * dir.x, pt.y + x[i] * dir.y, pt.z + x[i] * dir.z);
    const D3 norm = r0;
    r0.z          = 0.;
    const double inv = 1. / sqrt(r0.x * r0.x + r0.y * r0.y + r0.z * r0.z);
    r0               = d3(r0.x * inv, r0.y * inv, r0.z * inv);
    r0               = d3(r0.x * rtor, r0.y * rtor, r0.z * rtor);
    const double ndotd = (norm.x - r0.x) * dir.x + (norm.y - r0.y) * dir.y + (norm.z - r0.z) * dir.z;
    if (inner ^ out) {
      if (ndotd < 0) continue;
    } else {
      if (ndotd > 0) continue;
    }
    if (torus_has_phi(t)) {
      bool cin = false, cout = false;
      wedge_ci<true>(t + tr::TorWedge, r0, cin, cout);  // Wedge::ContainsWithBoundary
      if (cout) continue;
    }
    double s     = x[i];
    double eps   = kInfLength;
    double delta = s * s * s * s + a * s * s * s + b * s * s + c * s + d;
    double eps0  = -delta / (4. * s * s * s + 3. * a * s * s + 2. * b * s + c);
    int ntry     = 0;
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

// DistSqrToTorusR (TorusImplementation2.h:149-156)
__device__ __forceinline__ double torus_dist2_axis(const double *t, D3 p, D3 dir, double dist)
{
  const D3 q       = d3(p.x + dist * dir.x, p.y + dist * dir.y, p.z + dist * dir.z);
  const double rxy = sqrt(q.x * q.x + q.y * q.y);
  return (rxy - t[tr::TorRtor]) * (rxy - t[tr::TorRtor]) + q.z * q.z;
}

// Contains (TorusImplementation2.h:391-399): inside tolerances and no phi test, as the reference
__device__ __noinline__ bool torus_contains(const double *t, D3 p)
{
  bool cin = false, cout = false;
  torus_ci<true, false>(t, p, cin, cout);
  return !cout;
}

__device__ __noinline__ int torus_inside(const double *t, D3 p) { return torus_inside_kernel(t, p); }

// DistanceToIn (TorusImplementation2.h:415-491), the VECGEOM_NO_SPECIALIZATION branch
__device__ __noinline__ double torus_dist_in(const double *t, D3 p, D3 d)
{
  const double *bt   = t + tr::TorTube;
  const bool inBounds = tube_contains(bt, p);
  const double tubeDistance = inBounds ? 0. : tube_dist_in(bt, p, d);
  if (inBounds) {
    if (torus_inside_kernel(t, p) == kInsideE) return -1.;
  } else if (tubeDistance == kInfLength) {
    return kInfLength;
  }
  const D3 lp     = d3(p.x + tubeDistance * d.x, p.y + tubeDistance * d.y, p.z + tubeDistance * d.z);
  double distance = kInfLength;
  if (torus_has_phi(t)) {
    double d1, d2;
    wedge_dist<true>(t + tr::TorWedge, lp, d, d1, d2);
    if (d1 != kInfLength) {
      const double daxis = torus_dist2_axis(t, lp, d, d1);
      if (daxis >= t[tr::TorRmin2] && daxis < t[tr::TorRmax2]) {
        distance = d1;
        if (fabs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    if (d2 != kInfLength) {
      const double daxis = torus_dist2_axis(t, lp, d, d2);
      if (daxis >= t[tr::TorRmin2] && daxis < t[tr::TorRmax2]) {
        distance = d2 < distance ? d2 : distance;
        if (fabs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    distance = kInfLength;
  }
  double dd = torus_to_boundary(t, lp, d, t[tr::TorRmax], false);
  if (t[tr::TorRmin] > 0.) {
    const double ddrmin = torus_to_boundary(t, lp, d, t[tr::TorRmin], false);
    dd                  = dd < ddrmin ? dd : ddrmin;
  }
  distance = distance < dd ? distance : dd;
  distance += tubeDistance;
  if (fabs(distance) > kInfLength) distance = kInfLength;
  return distance;
}

// DistanceToOut (TorusImplementation2.h:158-217)
__device__ __noinline__ double torus_dist_out(const double *t, D3 p, D3 d)
{
  const double rtor = t[tr::TorRtor], rmax = t[tr::TorRmax];
  const double rsq       = p.x * p.x + p.y * p.y;
  const double outerExcl = rtor + rmax + kHalfTolerance, innerExcl = rtor - rmax - kHalfTolerance;
  if (fabs(p.z) - rmax > kHalfTolerance || rsq > outerExcl * outerExcl || rsq < innerExcl * innerExcl) return -1.;
  if (torus_inside_kernel(t, p) == kOutsideE) return -1.;
  const double dout = torus_to_boundary(t, p, d, rmax, true);
  double din        = kInfLength;
  if (t[tr::TorRmin] > 0) din = torus_to_boundary(t, p, d, t[tr::TorRmin], true);
  double distance = dout < din ? dout : din;
  if (torus_has_phi(t)) {
    const double *w = t + tr::TorWedge;
    double dp1, dp2;
    wedge_dist<false>(w, p, d, dp1, dp2);
    if (dp1 < distance) {
      const D3 ip = d3(p.x + dp1 * d.x, p.y + dp1 * d.y, p.z + dp1 * d.z);
      if (torus_contains_disk(t, ip)) {
        const double diri = ip.x * w[row::WedgeA1x] + ip.y * w[row::WedgeA1y];
        if (diri >= 0) distance = dp1;
      }
    }
    if (dp2 < distance) {
      const D3 ip = d3(p.x + dp2 * d.x, p.y + dp2 * d.y, p.z + dp2 * d.z);
      if (torus_contains_disk(t, ip)) {
        const double diri2 = ip.x * w[row::WedgeA2x] + ip.y * w[row::WedgeA2y];
        if (diri2 >= 0 && dp2 < distance) distance = dp2;
      }
    }
  }
  if (distance >= kInfLength) distance = -1.;
  return distance;
}

// SafetyToIn (TorusImplementation2.h:493-509)
__device__ __noinline__ double torus_safe_in(const double *t, D3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t[tr::TorRtor]) * (rxy - t[tr::TorRtor]) + p.z * p.z);
  double safety    = rad - t[tr::TorRmax];
  if (t[tr::TorRmin] != 0.) safety = vmax(t[tr::TorRmin] - rad, rad - t[tr::TorRmax]);
  if (torus_has_phi(t) && rxy != 0.) safety = vmax(wedge_safe_in(t + tr::TorWedge, p), safety);
  return safety;
}

// SafetyToOut (TorusImplementation2.h:379-389)
__device__ __noinline__ double torus_safe_out(const double *t, D3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t[tr::TorRtor]) * (rxy - t[tr::TorRtor]) + p.z * p.z);
  double safety    = t[tr::TorRmax] - rad;
  if (t[tr::TorRmin] != 0.) safety = vmin(rad - t[tr::TorRmin], t[tr::TorRmax] - rad);
  if (torus_has_phi(t)) safety = vmin(wedge_safe_out(t + tr::TorWedge, p), safety);
  return safety;
}
#endif  // VGN_SECTIONS

// ---------------------------------------------------------------- dispatch (primitive shapes)
// `stepmax` is the step the caller still accepts; of the primitives only the cut tube's DistanceToIn
// reads it (booleans hand it to their operands)
__device__ __forceinline__ double prim_dist_in(int type, const double *r, D3 p, D3 d, double stepmax)
{
  switch (type) {
  case kBox: return box_dist_in(r, p, d);
  case kTube: return tube_dist_in(r, p, d);
  case kCone: return cone_dist_in(r, p, d);
  case kTrd: return trd_dist_in(r, p, d);
  case kTrapezoid: return trap_dist_in(r, p, d);
  case kSphere: return sphere_dist_in(r, p, d);
  case kPolycone: return pcon_dist_in(r, p, d);
  case kOrb: return orb_dist_in(r, p, d);
  case kCutTube: return cuttube_dist_in(r, p, d, stepmax);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_dist_in(r, p, d);
  case kTorus: return torus_dist_in(r, p, d);
#endif
  }
  return kInfLength;
}

__device__ __forceinline__ double prim_dist_out(int type, const double *r, D3 p, D3 d)
{
  switch (type) {
  case kBox: return box_dist_out(r, p, d);
  case kTube: return tube_dist_out(r, p, d);
  case kCone: return cone_dist_out(r, p, d);
  case kTrd: return trd_dist_out(r, p, d);
  case kTrapezoid: return trap_dist_out(r, p, d);
  case kSphere: return sphere_dist_out(r, p, d);
  case kPolycone: return pcon_dist_out(r, p, d);
  case kOrb: return orb_dist_out(r, p, d);
  case kCutTube: return cuttube_dist_out(r, p, d);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_dist_out(r, p, d);
  case kTorus: return torus_dist_out(r, p, d);
#endif
  }
  return -1.;
}

__device__ __forceinline__ double prim_safe_in(int type, const double *r, D3 p)
{
  switch (type) {
  case kBox: return box_safe_in(r, p);
  case kTube: return tube_safe_in(r, p);
  case kCone: return cone_safe_in(r, p);
  case kTrd: return trd_safe_in(r, p);
  case kTrapezoid: return trap_safe_in(r, p);
  case kSphere: return sphere_safe_in(r, p);
  case kPolycone: return pcon_safe_in(r, p);
  case kOrb: return orb_safe_in(r, p);
  case kCutTube: return cuttube_safe_in(r, p);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_safety(r, p, false);
  case kTorus: return torus_safe_in(r, p);
#endif
  }
  return kInfLength;
}

__device__ __forceinline__ double prim_safe_out(int type, const double *r, D3 p)
{
  switch (type) {
  case kBox: return box_safe_out(r, p);
  case kTube: return tube_safe_out(r, p);
  case kCone: return cone_safe_out(r, p);
  case kTrd: return trd_safe_out(r, p);
  case kTrapezoid: return trap_safe_out(r, p);
  case kSphere: return sphere_safe_out(r, p);
  case kPolycone: return pcon_safe_out(r, p);
  case kOrb: return orb_safe_out(r, p);
  case kCutTube: return cuttube_safe_out(r, p);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_safety(r, p, true);
  case kTorus: return torus_safe_out(r, p);
#endif
  }
  return 0.;
}

__device__ __forceinline__ bool prim_contains(int type, const double *r, D3 p)
{
  switch (type) {
  case kBox: return box_contains(r, p);
  case kTube: return tube_contains(r, p);
  case kCone: return cone_contains(r, p);
  case kTrd: return trd_contains(r, p);
  case kTrapezoid: return trap_contains(r, p);
  case kSphere: return sphere_contains(r, p);
  case kPolycone: return pcon_contains(r, p);
  case kOrb: return orb_contains(r, p);
  case kCutTube: return cuttube_contains(r, p);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_contains(r, p);
  case kTorus: return torus_contains(r, p);
#endif
  }
  return false;
}

__device__ __forceinline__ int prim_inside(int type, const double *r, D3 p)
{
  switch (type) {
  case kBox: return box_inside(r, p);
  case kTube: return tube_inside(r, p);
  case kCone: return cone_inside(r, p);
  case kTrd: return trd_inside(r, p);
  case kTrapezoid: return trap_inside(r, p);
  case kSphere: return sphere_inside(r, p);
  case kPolycone: return pcon_inside(r, p);
  case kOrb: return orb_inside(r, p);
  case kCutTube: return cuttube_inside(r, p);
#if VGN_SECTIONS
  case kPolyhedron: return polyhedron_inside(r, p);
  case kTorus: return torus_inside(r, p);
#endif
  }
  return kOutsideE;
}

#if VGN_BOOLEANS
// ---------------------------------------------------------------- Boolean solids
// BooleanImplementation.h (subtraction), BooleanUnionImplementation.h and
// BooleanIntersectionImplementation.h over placed operands.  A placed operand's Contains,
// Inside, DistanceToIn, PlacedDistanceToOut and SafetyToIn take the boolean-frame point into the
// operand's frame (SpecializedPlacedVolImplHelper.h:99-172); its DistanceToOut and SafetyToOut
// do not (PlacedVolImplHelper.h:76-100).  Operands are primitives or (DEPTH 2) booleans of
// primitives.  The reference's loops are unbounded; these stop after kBoolMaxIter rounds
// (never reached on a valid solid).  Out of line: a boolean's code holds the operands' shape
// dispatch several times over and is needed only where booleans are placed.
constexpr long kBoolMaxIter = 1000000;

struct BoolOperand {
  int type;
  const double *row, *t, *r;  // shape row, placement translation and rotation
};
__device__ __forceinline__ BoolOperand bool_operand(const double *b, int k)
{
  const int ti = k == 0 ? row::BoolLeftType : row::BoolRightType;
  const int ri = k == 0 ? row::BoolLeftRow : row::BoolRightRow;
  const double *x = b + (k == 0 ? row::BoolLeftXf : row::BoolRightXf);
  return BoolOperand{(int)b[ti], b + (long)b[ri], x, x + 3};
}
__device__ __forceinline__ D3 axpy(D3 p, double a, D3 d) { return d3(p.x + a * d.x, p.y + a * d.y, p.z + a * d.z); }

template <int DEPTH> __device__ __noinline__ bool bool_contains(const double *b, D3 p);
template <int DEPTH> __device__ __noinline__ int bool_inside(const double *b, D3 p);
template <int DEPTH> __device__ __noinline__ double bool_dist_in(const double *b, D3 p, D3 d, double stepmax);
template <int DEPTH> __device__ __noinline__ double bool_dist_out(const double *b, D3 p, D3 d, double stepmax);
template <int DEPTH> __device__ __noinline__ double bool_safe_in(const double *b, D3 p);
template <int DEPTH> __device__ __noinline__ double bool_safe_out(const double *b, D3 p);

// the primitive dispatch for the booleans' operands, once each, out of line
__device__ __noinline__ bool prim_contains_ool(int type, const double *r, D3 p) { return prim_contains(type, r, p); }
__device__ __noinline__ int prim_inside_ool(int type, const double *r, D3 p) { return prim_inside(type, r, p); }
__device__ __noinline__ double prim_dist_in_ool(int type, const double *r, D3 p, D3 d, double stepmax)
{
  return prim_dist_in(type, r, p, d, stepmax);
}
__device__ __noinline__ double prim_dist_out_ool(int type, const double *r, D3 p, D3 d)
{
  return prim_dist_out(type, r, p, d);
}
__device__ __noinline__ double prim_safe_in_ool(int type, const double *r, D3 p) { return prim_safe_in(type, r, p); }
__device__ __noinline__ double prim_safe_out_ool(int type, const double *r, D3 p) { return prim_safe_out(type, r, p); }

// an operand's unplaced queries: a primitive, or at DEPTH 2 a boolean of primitives
template <int DEPTH>
__device__ __forceinline__ bool op_contains(int type, const double *r, D3 p)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_contains<DEPTH - 1>(r, p);
  }
  return prim_contains_ool(type, r, p);
}
template <int DEPTH>
__device__ __forceinline__ int op_inside(int type, const double *r, D3 p)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_inside<DEPTH - 1>(r, p);
  }
  return prim_inside_ool(type, r, p);
}
template <int DEPTH>
__device__ __forceinline__ double op_dist_in(int type, const double *r, D3 p, D3 d, double stepmax)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_dist_in<DEPTH - 1>(r, p, d, stepmax);
  }
  return prim_dist_in_ool(type, r, p, d, stepmax);
}
template <int DEPTH>
__device__ __forceinline__ double op_dist_out(int type, const double *r, D3 p, D3 d, double stepmax)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_dist_out<DEPTH - 1>(r, p, d, stepmax);
  }
  return prim_dist_out_ool(type, r, p, d);
}
template <int DEPTH>
__device__ __forceinline__ double op_safe_in(int type, const double *r, D3 p)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_safe_in<DEPTH - 1>(r, p);
  }
  return prim_safe_in_ool(type, r, p);
}
template <int DEPTH>
__device__ __forceinline__ double op_safe_out(int type, const double *r, D3 p)
{
  if constexpr (DEPTH > 1) {
    if (type == kBoolean) return bool_safe_out<DEPTH - 1>(r, p);
  }
  return prim_safe_out_ool(type, r, p);
}
// placed forms
template <int DEPTH>
__device__ __forceinline__ bool pl_contains(const BoolOperand &o, D3 p)
{
  return op_contains<DEPTH>(o.type, o.row, xf_point(o.t, o.r, p));
}
template <int DEPTH>
__device__ __forceinline__ int pl_inside(const BoolOperand &o, D3 p)
{
  return op_inside<DEPTH>(o.type, o.row, xf_point(o.t, o.r, p));
}
template <int DEPTH>
__device__ __forceinline__ double pl_dist_in(const BoolOperand &o, D3 p, D3 d, double stepmax)
{
  return op_dist_in<DEPTH>(o.type, o.row, xf_point(o.t, o.r, p), xf_dir(o.r, d), stepmax);
}
template <int DEPTH>
__device__ __forceinline__ double pl_dist_out(const BoolOperand &o, D3 p, D3 d, double stepmax)
{
  return op_dist_out<DEPTH>(o.type, o.row, xf_point(o.t, o.r, p), xf_dir(o.r, d), stepmax);
}
template <int DEPTH>
__device__ __forceinline__ double pl_safe_in(const BoolOperand &o, D3 p)
{
  return op_safe_in<DEPTH>(o.type, o.row, xf_point(o.t, o.r, p));
}

template <int DEPTH>
__device__ __noinline__ bool bool_contains(const double *b, D3 p)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  switch ((int)b[row::BoolOp]) {
  case 0:  // BooleanUnionImplementation.h Contains
    if (pl_contains<DEPTH>(L, p)) return true;
    return pl_contains<DEPTH>(R, p);
  case 1: {  // BooleanIntersectionImplementation.h Contains
    const bool a = pl_contains<DEPTH>(L, p);
    const bool r = pl_contains<DEPTH>(R, p);
    return a && r;
  }
  default:  // BooleanImplementation.h Contains
    if (!pl_contains<DEPTH>(L, p)) return false;
    return !pl_contains<DEPTH>(R, p);
  }
}

// kSurfaceE on both operands of a union takes their normals: answered -1 (not supported)
template <int DEPTH>
__device__ __noinline__ int bool_inside(const double *b, D3 p)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  const int a = pl_inside<DEPTH>(L, p);
  int r;
  switch ((int)b[row::BoolOp]) {
  case 0:
    if (a == kInsideE) return kInsideE;
    r = pl_inside<DEPTH>(R, p);
    if (r == kInsideE) return kInsideE;
    if (a == kSurfaceE && r == kSurfaceE) return -1;
    if (r == kSurfaceE || a == kSurfaceE) return kSurfaceE;
    return kOutsideE;
  case 1:
    if (a == kOutsideE) return kOutsideE;
    r = pl_inside<DEPTH>(R, p);
    if (a == kInsideE && r == kInsideE) return kInsideE;
    if ((a == kInsideE && r == kSurfaceE) || (r == kInsideE && a == kSurfaceE) || (a == kSurfaceE && r == kSurfaceE))
      return kSurfaceE;
    return kOutsideE;
  default:
    if (a == kOutsideE) return kOutsideE;
    r = pl_inside<DEPTH>(R, p);
    if (a == kInsideE && r == kOutsideE) return kInsideE;
    if ((a == kInsideE && r == kSurfaceE) || (r == kOutsideE && a == kSurfaceE)) return kSurfaceE;
    return kOutsideE;
  }
}

template <int DEPTH>
__device__ __noinline__ double bool_dist_in(const double *b, D3 p, D3 d, double stepmax)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  const int op = (int)b[row::BoolOp];
  if (op == 0) {
    const double d1 = pl_dist_in<DEPTH>(L, p, d, stepmax);
    const double d2 = pl_dist_in<DEPTH>(R, p, d, stepmax);
    return vmin(d1, d2);
  }
  if (op == 1) {
    D3 hit       = p;
    bool inleft  = pl_contains<DEPTH>(L, hit);
    bool inright = pl_contains<DEPTH>(R, hit);
    double d1 = 0., d2 = 0., snext = 0.;
    if (inleft && inright) {
      d1 = pl_dist_out<DEPTH>(L, hit, d, stepmax);
      d2 = pl_dist_out<DEPTH>(R, hit, d, stepmax);
      if (d1 < 2 * kTolerance) inleft = false;
      if (d2 < 2 * kTolerance) inright = false;
      if (inleft && inright) return 0.0;
    }
    for (long it = 0; it < kBoolMaxIter; ++it) {
      d1 = d2 = 0;
      if (!inleft) {
        d1 = vmax(pl_dist_in<DEPTH>(L, hit, d, kInfLength), kTolerance);
        if (d1 > 1E20) return kInfLength;
      }
      if (!inright) {
        d2 = vmax(pl_dist_in<DEPTH>(R, hit, d, kInfLength), kTolerance);
        if (d2 > 1E20) return kInfLength;
      }
      if (d1 > d2) {
        snext += d1;
        inleft  = true;
        hit     = axpy(hit, d1, d);
        inright = pl_contains<DEPTH>(R, axpy(hit, kTolerance, d));
        if (inright) return snext;
      } else {
        snext += d2;
        inright = true;
        hit     = axpy(hit, d2, d);
        inleft  = pl_contains<DEPTH>(L, axpy(hit, kTolerance, d));
        if (inleft) return snext;
      }
    }
    return kInfLength;
  }
  double d1, d2, snxt = 0.;
  D3 hit             = p;
  bool insideRight   = pl_contains<DEPTH>(R, p);
  const double epsil = kPushTolerance;
  for (long it = 0; it < kBoolMaxIter; ++it) {
    if (insideRight) {
      d1 = pl_dist_out<DEPTH>(R, hit, d, stepmax);
      snxt += (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : 0.;
      hit = axpy(hit, (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : 0., d);
      if (pl_contains<DEPTH>(L, hit)) {
        const double check = pl_dist_out<DEPTH>(L, hit, d, kInfLength);
        if (check > epsil) return snxt;
      }
    }
    d2 = vmax(pl_dist_in<DEPTH>(L, hit, d, stepmax), 0.);
    if (d2 == kInfLength) return kInfLength;
    d1 = pl_dist_in<DEPTH>(R, hit, d, stepmax);
    if (d2 < d1 - kTolerance) {
      snxt += d2 + epsil;
      return snxt;
    }
    snxt += (d1 >= 0. && d1 < kInfLength) ? d1 + epsil : 0.;
    hit         = axpy(hit, (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : epsil, d);
    insideRight = true;
  }
  return kInfLength;
}

// BooleanUnionImplementation.h DistanceToOut: the walk over connecting operands
template <int DEPTH>
__device__ __forceinline__ double union_out_walk(const BoolOperand &A, const BoolOperand &B, D3 p, D3 d)
{
  double dist           = 0.;
  const double pushdist = kPushTolerance;
  D3 nextp              = p;
  bool connecting;
  long it = 0;
  do {
    connecting    = false;
    double disTmp = pl_dist_out<DEPTH>(A, nextp, d, kInfLength);
    dist += (disTmp >= 0. && disTmp < kInfLength) ? disTmp : 0;
    dist += pushdist;
    nextp = axpy(p, dist, d);
    if (pl_inside<DEPTH>(B, nextp) != kOutsideE) {
      disTmp = pl_dist_out<DEPTH>(B, nextp, d, kInfLength);
      dist += (disTmp >= 0. && disTmp < kInfLength) ? disTmp : 0;
      dist += pushdist;
      nextp      = axpy(p, dist, d);
      connecting = true;
    }
  } while (connecting && pl_inside<DEPTH>(A, nextp) != kOutsideE && ++it < kBoolMaxIter);
  return dist;
}

template <int DEPTH>
__device__ __noinline__ double bool_dist_out(const double *b, D3 p, D3 d, double stepmax)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  const int op = (int)b[row::BoolOp];
  if (op == 0) {
    const int posA    = pl_inside<DEPTH>(L, p);
    const double dist = posA != kOutsideE ? union_out_walk<DEPTH>(L, R, p, d) : union_out_walk<DEPTH>(R, L, p, d);
    double distance   = dist - kPushTolerance;
    if (distance < kTolerance && posA == kOutsideE && pl_inside<DEPTH>(R, p) == kOutsideE) distance = -kTolerance;
    return distance;
  }
  if (op == 1) {
    const double a = op_dist_out<DEPTH>(L.type, L.row, p, d, kInfLength);  // the left operand unplaced
    const double r = pl_dist_out<DEPTH>(R, p, d, kInfLength);
    return vmin(a, r);
  }
  const double distancel = pl_dist_out<DEPTH>(L, p, d, stepmax);
  const double dinright  = pl_dist_in<DEPTH>(R, p, d, stepmax);
  return vmin(distancel, dinright);
}

template <int DEPTH>
__device__ __noinline__ double bool_safe_in(const double *b, D3 p)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  const int op = (int)b[row::BoolOp];
  if (op == 0) return vmin(pl_safe_in<DEPTH>(L, p), pl_safe_in<DEPTH>(R, p));
  if (op == 1) {
    const bool insideA = pl_contains<DEPTH>(L, p);
    const bool insideB = pl_contains<DEPTH>(R, p);
    if (!insideA && insideB) return pl_safe_in<DEPTH>(L, p);
    if (!insideB && insideA) return pl_safe_in<DEPTH>(R, p);
    return vmin(pl_safe_in<DEPTH>(L, p), pl_safe_in<DEPTH>(R, p));
  }
  if (pl_contains<DEPTH>(L, p) && pl_contains<DEPTH>(R, p)) return op_safe_out<DEPTH>(R.type, R.row, xf_point(R.t, R.r, p));
  return pl_safe_in<DEPTH>(L, p);
}

template <int DEPTH>
__device__ __noinline__ double bool_safe_out(const double *b, D3 p)
{
  const BoolOperand L = bool_operand(b, 0), R = bool_operand(b, 1);
  const int op = (int)b[row::BoolOp];
  if (op == 0) {
    const int insideA = pl_inside<DEPTH>(L, p);
    const int insideB = pl_inside<DEPTH>(R, p);
    if (insideA == kOutsideE && insideB == kOutsideE) return -kTolerance;
    if (insideA != kOutsideE && insideB != kOutsideE)
      return vmax(op_safe_out<DEPTH>(L.type, L.row, p), op_safe_out<DEPTH>(R.type, R.row, xf_point(R.t, R.r, p)));
    if (insideA == kSurfaceE || insideB == kSurfaceE) return -kTolerance;
    if (insideA == kOutsideE) return op_safe_out<DEPTH>(R.type, R.row, xf_point(R.t, R.r, p));
    return op_safe_out<DEPTH>(L.type, L.row, p);
  }
  if (op == 1) {
    double safety = vmin(op_safe_out<DEPTH>(L.type, L.row, p), op_safe_out<DEPTH>(R.type, R.row, xf_point(R.t, R.r, p)));
    if (safety < 0.) safety = 0.;
    return safety;
  }
  return vmin(op_safe_out<DEPTH>(L.type, L.row, p), pl_safe_in<DEPTH>(R, p));
}

#endif  // VGN_BOOLEANS

// ---------------------------------------------------------------- dispatch (all shape types)
// `stepmax` is the step the caller still accepts (the BVH passes its running step, BVH.h:115;
// the navigator its step limit to the mother's DistanceToOut, VNavigator.h:246): the cut tube's
// DistanceToIn and the booleans use it.  Kernel sets without the boolean code dispatch the
// primitives only (the host runs geometries with booleans on the `booleans` set).
#if VGN_BOOLEANS
#define VGN_BOOL_OR(call, prim) (type == kBoolean ? call : prim)
#else
#define VGN_BOOL_OR(call, prim) (prim)
#endif
__device__ __forceinline__ double shape_dist_in(int type, const double *r, D3 p, D3 d, double stepmax = kInfLength)
{
  return VGN_BOOL_OR((bool_dist_in<2>(r, p, d, stepmax)), (prim_dist_in(type, r, p, d, stepmax)));
}
__device__ __forceinline__ double shape_dist_out(int type, const double *r, D3 p, D3 d, double stepmax = kInfLength)
{
  (void)stepmax;
  return VGN_BOOL_OR((bool_dist_out<2>(r, p, d, stepmax)), (prim_dist_out(type, r, p, d)));
}
__device__ __forceinline__ double shape_safe_in(int type, const double *r, D3 p)
{
  return VGN_BOOL_OR((bool_safe_in<2>(r, p)), (prim_safe_in(type, r, p)));
}
__device__ __forceinline__ double shape_safe_out(int type, const double *r, D3 p)
{
  return VGN_BOOL_OR((bool_safe_out<2>(r, p)), (prim_safe_out(type, r, p)));
}
__device__ __forceinline__ bool shape_contains(int type, const double *r, D3 p)
{
  return VGN_BOOL_OR((bool_contains<2>(r, p)), (prim_contains(type, r, p)));
}
__device__ __forceinline__ int shape_inside(int type, const double *r, D3 p)
{
  return VGN_BOOL_OR((bool_inside<2>(r, p)), (prim_inside(type, r, p)));
}
#undef VGN_BOOL_OR

}  // namespace VGN_KSET
}  // namespace dev
}  // namespace vgn
