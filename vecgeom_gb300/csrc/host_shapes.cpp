// host_shapes.cpp -- shape parameter rows and extents (host side).
//
// A row holds the shape's defining parameters plus the cached members the
// reference precomputes in its *Struct constructors, computed with the same
// expressions so the device kernels see the same doubles.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "../../include/vgnav.h"
#include "host_geometry.h"

namespace vgn {

static constexpr double kTolerance     = 1e-9;
static constexpr double kHalfTolerance = 0.5 * kTolerance;
static constexpr double kPi            = 3.14159265358979323846;
static constexpr double kTwoPi         = 2. * kPi;
static constexpr double kConeTolerance = 1e-7;
static constexpr double kAngTolerance  = 1e-9;

static inline double nonzero(double x) { return x + std::copysign(1.0e-30, x); }  // Global.h:174-178

// evolution::Wedge(angle = dphi, zeroangle = sphi) (source/Wedge_Evolution.cpp:17-99) into a
// row::Wedge* block
static void wedge_fill(double *w, double dphi, double sphi)
{
  w[row::WedgeA1x]  = std::cos(sphi);
  w[row::WedgeA1y]  = std::sin(sphi);
  w[row::WedgeA2x]  = std::cos(sphi + dphi);
  w[row::WedgeA2y]  = std::sin(sphi + dphi);
  w[row::WedgeN1x]  = -std::sin(sphi);
  w[row::WedgeN1y]  = std::cos(sphi);
  w[row::WedgeN2x]  = std::sin(sphi + dphi);
  w[row::WedgeN2y]  = -std::cos(sphi + dphi);
  w[row::WedgeDPhi] = dphi;
}

// Wedge::Contains: !completelyoutside of GenericKernelForContainsAndInside<false>
// (Wedge_Evolution.h:296-339) at a point of the z = 0 plane
static bool wedge_contains(const double *w, double x, double y)
{
  const double startCheck = (-x * w[row::WedgeA1y] + y * w[row::WedgeA1x]);
  const double endCheck   = (-w[row::WedgeA2x] * y + w[row::WedgeA2y] * x);
  bool out                = startCheck < 0.;
  if (w[row::WedgeDPhi] < kPi)
    out = out || endCheck < 0.;
  else
    out = out && endCheck < 0.;
  return !out;
}

int shape_param_count(int32_t type, const double *p, int32_t n_avail)
{
  switch (type) {
  case kBox: return 3;
  case kTube: return 5;
  case kCone: return 7;
  case kTrd: return 5;
  case kTrapezoid: return 11;
  case kSphere: return 6;
  case kOrb: return 1;
  case kCutTube: return 11;
  case kBoolean: return 3;  // operation, left and right operand placements
  case kPolycone: {  // sphi, dphi, nz, z[nz], rmin[nz], rmax[nz]
    if (n_avail < 3 || !(p[2] >= 2 && p[2] <= 4096) || (double)(int)p[2] != p[2]) return -1;
    return 3 + 3 * (int)p[2];
  }
  case kTorus: return 5;
  case kPolyhedron: {  // sphi, dphi, sides, nz, z[nz], rmin[nz], rmax[nz]
    if (n_avail < 4 || !(p[3] >= 2 && p[3] <= 4096) || (double)(int)p[3] != p[3]) return -1;
    if (!(p[2] >= 1 && p[2] <= 4096) || (double)(int)p[2] != p[2]) return -1;
    return 4 + 3 * (int)p[3];
  }
  default: return -1;
  }
}

// ---------------------------------------------------------------- Polyhedron
// PolyhedronStruct(phiStart, phiDelta, sideCount, zPlaneCount, zPlanes, rMin, rMax) and
// Initialize (PolyhedronStruct.h:96-110, 264-420), Quadrilaterals::Set (source/Quadrilaterals.cpp:33-104),
// Planes::Set / FlipSign (source/Planes.cpp:30-49), in the row layout row::Phd*.
namespace {
struct PV3 {
  double x, y, z;
};
inline PV3 pv3(double x, double y, double z) { return PV3{x, y, z}; }
inline PV3 operator-(PV3 a, PV3 b) { return pv3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline double pdot(PV3 a, PV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline PV3 pcross(PV3 a, PV3 b) { return pv3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline PV3 pfix(PV3 a)  // Vector3D::FixZeroes (Vector3D.h:298-305)
{
  if (std::fabs(a.x) < kTolerance) a.x = 0.0;
  if (std::fabs(a.y) < kTolerance) a.y = 0.0;
  if (std::fabs(a.z) < kTolerance) a.z = 0.0;
  return a;
}
inline PV3 pnormalized(PV3 a)  // Vector3D::Normalized (Vector3D.h:202)
{
  const double inv = 1. / std::sqrt(pdot(a, a));
  return pv3(a.x * inv, a.y * inv, a.z * inv);
}
inline bool ptol_eq(PV3 a, PV3 b)  // operator== (Vector3D.h:387-390)
{
  return std::fabs(a.x - b.x) < kTolerance && std::fabs(a.y - b.y) < kTolerance && std::fabs(a.z - b.z) < kTolerance;
}
inline double phd_normalize_angle(double a) { return a + kTwoPi * (double)((a < 0) - (int)(a / kTwoPi)); }

// Quadrilaterals::Set of one face into q[kQuadSize]; false when fewer than three corners differ
bool quad_set(double *q, const PV3 (&in)[4])
{
  PV3 ch[4];
  int assigned = 1;
  for (int j = 0; j < 4; ++j) {
    q[row::QuadCorner + 3 * j]     = in[j].x;
    q[row::QuadCorner + 3 * j + 1] = in[j].y;
    q[row::QuadCorner + 3 * j + 2] = in[j].z;
  }
  ch[0] = in[0];
  for (int tested = 1; tested < 4; ++tested) {
    bool chosen = true;
    for (int j = 0; j < assigned; ++j)
      if (ptol_eq(ch[j], in[tested])) {
        chosen = false;
        break;
      }
    if (chosen) ch[assigned++] = in[tested];
  }
  if (assigned < 3) return false;
  const double a = ch[0].y * (ch[1].z - ch[2].z) + ch[1].y * (ch[2].z - ch[0].z) + ch[2].y * (ch[0].z - ch[1].z);
  const double b = ch[0].z * (ch[1].x - ch[2].x) + ch[1].z * (ch[2].x - ch[0].x) + ch[2].z * (ch[0].x - ch[1].x);
  const double c = ch[0].x * (ch[1].y - ch[2].y) + ch[1].x * (ch[2].y - ch[0].y) + ch[2].x * (ch[0].y - ch[1].y);
  double d = -ch[0].x * (ch[1].y * ch[2].z - ch[2].y * ch[1].z) - ch[1].x * (ch[2].y * ch[0].z - ch[0].y * ch[2].z) -
             ch[2].x * (ch[0].y * ch[1].z - ch[1].y * ch[0].z);
  PV3 n            = pv3(a, b, c);
  const double inv = 1. / std::sqrt(pdot(n, n));
  n                = pv3(n.x * inv, n.y * inv, n.z * inv);
  d *= inv;
  n                  = pfix(n);
  q[row::QuadN]      = n.x;
  q[row::QuadN + 1]  = n.y;
  q[row::QuadN + 2]  = n.z;
  q[row::QuadD]      = d;
  for (int j = 0; j < 4; ++j) {
    double *s     = q + row::QuadSide + 4 * j;
    const PV3 c0 = in[j], c1 = in[(j + 1) % 4];
    if (!ptol_eq(c1, c0)) {
      const PV3 fixed   = pfix(pnormalized(pcross(n, c1 - c0)));
      const double sinv = 1. / std::sqrt(pdot(fixed, fixed));
      s[0]              = sinv * fixed.x;
      s[1]              = sinv * fixed.y;
      s[2]              = sinv * fixed.z;
      s[3]              = sinv * -pdot(fixed, c0);
    } else {
      s[0] = s[1] = s[2] = s[3] = 0.;
    }
  }
  return true;
}

void quad_flip(double *q)
{
  for (int k = 0; k < 4; ++k) q[k] = -q[k];  // normal and distance (QuadN .. QuadD)
}

int polyhedron_row(const double *p, std::vector<double> &shape, std::string &err)
{
  const double phiStart0 = p[0], phiDelta0 = p[1];
  const int S = (int)p[2], nz = (int)p[3];
  const double *zp = p + 4, *rmn = p + 4 + nz, *rmx = p + 4 + 2 * nz;
  if (!(phiDelta0 > 0) || S < 1 || nz < 2 || !((phiDelta0 > kTwoPi ? kTwoPi : phiDelta0) / S < kPi)) {
    err = "polyhedron needs dphi > 0, nz >= 2 and sides with dphi / sides < pi";
    return VGN_ERR_ARG;
  }
  for (int i = 0; i < nz; ++i) {
    if (!(rmn[i] >= 0 && rmx[i] >= rmn[i]) || (i > 0 && !(zp[i] >= zp[i - 1]))) {
      err = "polyhedron needs 0 <= rmin <= rmax and non-decreasing z planes";
      return VGN_ERR_ARG;
    }
    if (i + 2 < nz && zp[i] == zp[i + 1] && zp[i + 1] == zp[i + 2]) {
      err = "polyhedron has three equal z planes in a row";
      return VGN_ERR_ARG;
    }
  }
  if (zp[0] == zp[1] || zp[nz - 2] == zp[nz - 1]) {
    err = "polyhedron has a zero-length first or last segment";
    return VGN_ERR_ARG;
  }
  const bool hasPhi = phiDelta0 < kTwoPi;
  const double phiStart = phd_normalize_angle(phiStart0), phiDelta = phiDelta0 > kTwoPi ? kTwoPi : phiDelta0;
  const double sidePhi = phiDelta / S, cosHalf = std::cos(0.5 * sidePhi);
  // face counts per segment (Initialize, PolyhedronStruct.h:304-326)
  std::vector<int> nout(nz - 1), nphi(nz - 1), nin(nz - 1);
  for (int i = 0; i < nz - 1; ++i) {
    const bool hasInnerRadius = rmn[i] > 0 || rmn[i + 1] > 0;
    nout[i]                   = (zp[i] == zp[i + 1] && rmx[i] == rmx[i + 1]) ? 0 : S;
    nphi[i]                   = hasPhi ? (zp[i] == zp[i + 1] ? 0 : 2) : 0;
    nin[i]                    = (hasInnerRadius && !(zp[i] == zp[i + 1] && rmn[i] == rmn[i + 1])) ? S : 0;
    if (zp[i] == zp[i + 1] && nout[i] == 0 && nin[i] == 0) {
      err = "polyhedron has a zero-length segment with equal radii on its two planes";
      return VGN_ERR_ARG;
    }
  }
  const int segs  = row::phd_segs(nz, S);
  int nfaces      = 0;
  for (int i = 0; i < nz - 1; ++i) nfaces += nout[i] + nphi[i] + nin[i];
  std::vector<double> r((size_t)(segs + 4 * (nz - 1) + nfaces * row::kQuadSize), 0.);
  r[row::PhdSides]    = S;
  r[row::PhdNz]       = nz;
  r[row::PhdHasPhi]   = hasPhi ? 1. : 0.;
  r[row::PhdLargePhi] = phiDelta0 < kPi ? 1. : 0.;
  r[row::PhdPhiStart] = phiStart;
  r[row::PhdPhiDelta] = phiDelta;
  wedge_fill(&r[row::PhdWedge], phiDelta, phiStart);  // fPhiWedge(fPhiDelta, fPhiStart)
  for (int i = 0; i < nz; ++i) {
    r[row::phd_z(nz) + i]     = zp[i];
    r[row::phd_rmin(nz) + i]  = rmn[i];
    r[row::phd_rmax(nz) + i]  = rmx[i];
    r[row::phd_samez(nz) + i] = (i > 0 && i < nz - 1 && zp[i] == zp[i + 1]) ? 1. : 0.;
  }
  auto getPhi = [&](int side) { return phd_normalize_angle(phiStart + ((!hasPhi && side == S) ? 0 : side) * sidePhi); };
  PV3 phisec[2];
  for (int i = 0; i <= S; ++i) {
    const double phi = getPhi(i);
    const PV3 corner = pfix(pnormalized(pv3(1. * std::cos(phi), 1. * std::sin(phi), 0)));
    const PV3 s      = pcross(pnormalized(corner), pv3(0, 0, -1));
    r[row::phd_phisec(nz) + 3 * i]     = s.x;
    r[row::phd_phisec(nz) + 3 * i + 1] = s.y;
    r[row::phd_phisec(nz) + 3 * i + 2] = s.z;
    if (i == 0) phisec[0] = s;
    if (i == S) phisec[1] = s;
  }
  // the bounding tube (PolyhedronStruct.h:341-367)
  double inner = DBL_MAX, outer = -DBL_MAX;  // kInfLength
  for (int i = 0; i < nz; ++i) {
    if (rmn[i] < inner) inner = rmn[i];
    if (rmx[i] > outer) outer = rmx[i];
  }
  outer /= cosHalf;
  const double tp[5] = {inner - kHalfTolerance, outer + kHalfTolerance, 0.5 * (zp[nz - 1] - zp[0]) + kTolerance,
                        !hasPhi ? 0 : phiStart - 100 * kTolerance, !hasPhi ? kTwoPi : phiDelta + 2 * (100 * kTolerance)};
  std::vector<double> tube;
  if (int rc = shape_make_row(kTube, tp, 5, tube, err)) return rc;
  std::copy(tube.begin(), tube.end(), r.begin() + row::PhdTube);
  r[row::PhdTubeOffset] = 0.5 * (zp[0] + zp[nz - 1]);
  // the faces (PolyhedronStruct.h:369-418)
  auto vtx = [&](const double *rr, int i, int j) {
    const double phi = getPhi(j), R = rr[i] / cosHalf;
    return pfix(pv3(R * std::cos(phi), R * std::sin(phi), zp[i]));
  };
  int face = segs + 4 * (nz - 1);
  for (int ip = 0; ip < nz - 1; ++ip) {
    double *st = &r[segs + 4 * ip];
    st[0] = nout[ip];
    st[1] = nphi[ip];
    st[2] = nin[ip];
    st[3] = face;
    for (int k = 0; k < 2; ++k) {  // outer, then (after the phi faces) inner
      const double *rr = k == 0 ? rmx : rmn;
      const int n      = k == 0 ? nout[ip] : nin[ip];
      double *base     = &r[face + (k == 0 ? 0 : (nout[ip] + nphi[ip]) * row::kQuadSize)];
      for (int is = 0; is < n; ++is) {
        double *q           = base + is * row::kQuadSize;
        const PV3 corner[4] = {vtx(rr, ip, is), vtx(rr, ip, is + 1), vtx(rr, ip + 1, is + 1), vtx(rr, ip + 1, is)};
        if (!quad_set(q, corner)) {
          err = "polyhedron has a face with fewer than three distinct corners";
          return VGN_ERR_ARG;
        }
        if (q[0] * corner[0].x + q[1] * corner[0].y < 0) quad_flip(q);  // WrongNormal
      }
    }
    if (nphi[ip] == 2) {
      double *q0       = &r[face + nout[ip] * row::kQuadSize];
      double *q1       = q0 + row::kQuadSize;
      const PV3 c0[4]  = {vtx(rmn, ip, 0), vtx(rmn, ip + 1, 0), vtx(rmx, ip + 1, 0), vtx(rmx, ip, 0)};
      const PV3 c1[4]  = {vtx(rmx, ip, S), vtx(rmx, ip + 1, S), vtx(rmn, ip + 1, S), vtx(rmn, ip, S)};
      if (!quad_set(q0, c0) || !quad_set(q1, c1)) {
        err = "polyhedron has a face with fewer than three distinct corners";
        return VGN_ERR_ARG;
      }
      if (pdot(pv3(q0[0], q0[1], q0[2]), phisec[0]) > 0) quad_flip(q0);
      if (pdot(pv3(q1[0], q1[1], q1[2]), phisec[1]) < 0) quad_flip(q1);
    }
    face += (nout[ip] + nphi[ip] + nin[ip]) * row::kQuadSize;
  }
  shape.insert(shape.end(), r.begin(), r.end());
  return VGN_OK;
}
} // namespace

int shape_make_row(int32_t type, const double *p, int32_t n_avail, std::vector<double> &shape, std::string &err)
{
  (void)n_avail;
  switch (type) {
  case kBox: {
    // BoxStruct fDimensions (BoxStruct.h:19-27)
    if (!(p[0] > 0 && p[1] > 0 && p[2] > 0)) {
      err = "box half-lengths must be positive";
      return VGN_ERR_ARG;
    }
    shape.push_back(p[0]);
    shape.push_back(p[1]);
    shape.push_back(p[2]);
    shape.push_back(0.);
    return VGN_OK;
  }
  case kTube: {
    // TubeStruct(rmin, rmax, z, sphi, dphi) + CalculateCached (TubeStruct.h:43-72, 153-175);
    // the constructor keeps the raw (sphi, dphi) and builds its Wedge from them
    const double rmin = p[0] < 0.0 ? 0.0 : p[0], rmax = p[1], z = p[2], sphi = p[3], dphi = p[4];
    if (!(rmax > rmin && z > 0 && dphi > 0)) {
      err = "tube needs rmax > rmin, dz > 0 and dphi > 0";
      return VGN_ERR_ARG;
    }
    double row[row::kTubeSize];
    row[row::TubeSphi] = sphi;
    row[row::TubeTolOz] = z + kHalfTolerance;
    wedge_fill(row + row::TubeWedge, dphi, sphi);  // also fAlongPhi1/2 and fDphi
    row[row::TubeRmin] = rmin;
    row[row::TubeRmax] = rmax;
    row[row::TubeZ]    = z;
    row[row::TubeRmin2] = rmin * rmin;
    row[row::TubeRmax2] = rmax * rmax;
    const double tolOrmin = rmin - kHalfTolerance, tolIrmin = rmin + kHalfTolerance;
    const double tolOrmax = rmax + kHalfTolerance, tolIrmax = rmax - kHalfTolerance;
    row[row::TubeTolOrmin2] = tolOrmin * tolOrmin;
    row[row::TubeTolIrmin2] = tolIrmin * tolIrmin;
    row[row::TubeTolOrmax2] = tolOrmax * tolOrmax;
    row[row::TubeTolIrmax2] = tolIrmax * tolIrmax;
    row[row::TubeMaxVal]    = rmax > z ? rmax : z;
    shape.insert(shape.end(), row, row + row::kTubeSize);
    return VGN_OK;
  }
  case kCone: {
    // ConeStruct(rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi) + CalculateCached (ConeStruct.h:79-157, 414-426)
    double rmin1 = p[0] < 0.0 ? 0.0 : p[0], rmax1 = p[1], rmin2 = p[2] < 0.0 ? 0.0 : p[2], rmax2 = p[3];
    const double dz = p[4], sphi = p[5], dphi = p[6];
    if (!(dz > 0 && rmax1 >= rmin1 && rmax2 >= rmin2 && (rmax1 > 0 || rmax2 > 0) && dphi > 0)) {
      err = "cone needs dz > 0, rmax >= rmin at both ends and dphi > 0";
      return VGN_ERR_ARG;
    }
    double r[row::kConeSize];
    r[row::ConeArgRmax1]  = p[1];
    r[row::ConeArgRmax2]  = p[3];
    r[row::ConeArgRmin1]  = p[0];
    r[row::ConeArgRmin2]  = p[2];
    // fPhiWedge(_dphi, _sphi), then SetAndCheckDPhiAngle(_dphi) and SetAndCheckSPhiAngle(_sphi)
    // (ConeStruct.h:321-360, 413-425): the wedge keeps the raw angles' vectors and takes the
    // checked delta; the along vectors use the checked angles
    wedge_fill(r + row::ConeWedge, dphi, sphi);
    double cdphi = dphi, csphi = sphi;
    if (dphi >= kTwoPi - 0.5 * kAngTolerance) {
      cdphi = kTwoPi;
      csphi = 0;
    }
    r[row::ConeWedge + row::WedgeDPhi] = cdphi;
    if (sphi < 0)
      csphi = kTwoPi - std::fmod(std::fabs(sphi), kTwoPi);
    else
      csphi = std::fmod(sphi, kTwoPi);
    if (csphi + cdphi > kTwoPi) csphi -= kTwoPi;
    r[row::ConeSPhi] = csphi;
    r[row::ConeDPhi] = cdphi;
    r[row::ConeAP1x] = std::cos(csphi);
    r[row::ConeAP1y] = std::sin(csphi);
    r[row::ConeAP2x] = std::cos(csphi + cdphi);
    r[row::ConeAP2y] = std::sin(csphi + cdphi);
    r[row::ConeOrigRmax1] = rmax1;
    r[row::ConeOrigRmax2] = rmax2;
    if (rmin1 == rmax1) rmax1 += kConeTolerance;
    if (rmin2 == rmax2) rmax2 += kConeTolerance;
    r[row::ConeRmin1] = rmin1;
    r[row::ConeRmax1] = rmax1;
    r[row::ConeRmin2] = rmin2;
    r[row::ConeRmax2] = rmax2;
    r[row::ConeDz]    = dz;
    r[row::ConeSqRmin1] = rmin1 * rmin1;
    r[row::ConeSqRmax1] = rmax1 * rmax1;
    r[row::ConeSqRmin2] = rmin2 * rmin2;
    r[row::ConeSqRmax2] = rmax2 * rmax2;
    const double tanRMin = (rmin2 - rmin1) * 0.5 / dz;
    const double secRMin = std::sqrt(1.0 + tanRMin * tanRMin);
    const double tanRMax = (rmax2 - rmax1) * 0.5 / dz;
    const double secRMax = std::sqrt(1.0 + tanRMax * tanRMax);
    r[row::ConeTanRMin]    = tanRMin;
    r[row::ConeSecRMin]    = secRMin;
    r[row::ConeInvSecRMin] = 1. / nonzero(secRMin);
    r[row::ConeTanRMax]    = tanRMax;
    r[row::ConeSecRMax]    = secRMax;
    r[row::ConeInvSecRMax] = 1. / nonzero(secRMax);
    const double innerSlope = -(rmin1 - rmin2) / (2. * dz);
    const double outerSlope = -(rmax1 - rmax2) / (2. * dz);
    r[row::ConeInnerSlope]  = innerSlope;
    r[row::ConeOuterSlope]  = outerSlope;
    r[row::ConeInnerOffset] = rmin2 - innerSlope * dz;
    r[row::ConeOuterOffset] = rmax2 - outerSlope * dz;
    r[row::ConeInnerTol]    = kConeTolerance * secRMin;
    r[row::ConeOuterTol]    = kConeTolerance * secRMax;
    double innerApex, tanInner, outerApex, tanOuter;
    if (rmin2 > rmin1) {
      innerApex = 2 * dz * rmin1 / (rmin2 - rmin1);
      tanInner  = rmin2 / (2 * dz + innerApex);
    } else {
      innerApex = 2 * dz * rmin2 / nonzero(rmin1 - rmin2);
      tanInner  = rmin1 / (2 * dz + innerApex);
    }
    if (rmin1 == 0. || rmin2 == 0.) innerApex = 0.;
    if (rmin1 == 0.) tanInner = rmin2 / (2 * dz);
    if (rmin2 == 0.) tanInner = rmin1 / (2 * dz);
    if (rmax2 > rmax1) {
      outerApex = 2 * dz * rmax1 / (rmax2 - rmax1);
      tanOuter  = rmax2 / (2 * dz + outerApex);
    } else {
      outerApex = 2 * dz * rmax2 / nonzero(rmax1 - rmax2);
      tanOuter  = rmax1 / (2 * dz + outerApex);
    }
    if (rmax1 == 0. || rmax2 == 0.) outerApex = 0.;
    if (rmax1 == 0.) tanOuter = rmax2 / (2 * dz);
    if (rmax2 == 0.) tanOuter = rmax1 / (2 * dz);
    r[row::ConeInnerApex]    = innerApex;
    r[row::ConeTanInnerApex] = tanInner;
    r[row::ConeOuterApex]    = outerApex;
    r[row::ConeTanOuterApex] = tanOuter;
    r[row::ConeZNormInner]   = tanRMin / nonzero(secRMin);
    r[row::ConeZNormOuter]   = -tanRMax / nonzero(secRMax);
    r[row::ConeTolIz]        = dz - kHalfTolerance;
    shape.insert(shape.end(), r, r + row::kConeSize);
    return VGN_OK;
  }
  case kTrd: {
    // TrdStruct(x1, x2, y1, y2, z) + CalculateCached (TrdStruct.h:65-70, 103-119); the y
    // tolerance is computed from the x half-lengths, as the reference does
    if (!(p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[3] >= 0 && p[4] > 0)) {
      err = "Trd half-lengths must be >= 0 and dz > 0";
      return VGN_ERR_ARG;
    }
    double r[row::kTrdSize] = {};
    const double dx1 = p[0], dx2 = p[1], dy1 = p[2], dy2 = p[3], dz = p[4];
    const double fx = 0.5 * (dx1 - dx2) / dz, fy = 0.5 * (dy1 - dy2) / dz;
    const double x21         = dx2 - dx1;
    r[row::TrdDx1]          = dx1;
    r[row::TrdDx2]          = dx2;
    r[row::TrdDy1]          = dy1;
    r[row::TrdDy2]          = dy2;
    r[row::TrdDz]           = dz;
    r[row::TrdX2minusX1]    = x21;
    r[row::TrdY2minusY1]    = dy2 - dy1;
    r[row::TrdHalfX1plusX2] = 0.5 * (dx1 + dx2);
    r[row::TrdHalfY1plusY2] = 0.5 * (dy1 + dy2);
    r[row::TrdFx]           = fx;
    r[row::TrdFy]           = fy;
    r[row::TrdCalfX]        = 1. / std::sqrt(1.0 + fx * fx);
    r[row::TrdCalfY]        = 1. / std::sqrt(1.0 + fy * fy);
    r[row::TrdTolX]         = kTolerance * std::sqrt(x21 * x21 + 4 * dz * dz);
    r[row::TrdTolY]         = kTolerance * std::sqrt(x21 * x21 + 4 * dz * dz);
    shape.insert(shape.end(), r, r + row::kTrdSize);
    return VGN_OK;
  }
  case kTrapezoid: {
    // UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, Alpha1, dy2, dx3, dx4, Alpha2)
    // (UnplacedTrapezoid.h:56-64): tan of the alphas, CalculateCached (TrapezoidStruct.h:90-95),
    // corners from the parameters and one plane per side face
    // (source/UnplacedTrapezoid.cpp:447-466, 568-675)
    if (!(p[0] > 0 && p[3] > 0 && p[7] > 0 && p[4] >= 0 && p[5] >= 0 && p[8] >= 0 && p[9] >= 0 &&
          std::fabs(p[1]) < 0.5 * kPi)) {
      err = "Trapezoid needs dz, dy1, dy2 > 0, dx >= 0 and |theta| < pi/2";
      return VGN_ERR_ARG;
    }
    double r[row::kTrapSize] = {};
    const double dz = p[0], theta = p[1], phi = p[2], dy1 = p[3], dx1 = p[4], dx2 = p[5], dy2 = p[7], dx3 = p[8],
                 dx4 = p[9];
    const double tanA1 = std::tan(p[6]), tanA2 = std::tan(p[10]);
    const double tcp = std::tan(theta) * std::cos(phi), tsp = std::tan(theta) * std::sin(phi);
    const double dxdyDy1 = tanA1 * dy1, dxdyDy2 = tanA2 * dy2, dxdzDz = tcp * dz, dydzDz = tsp * dz;
    const Vec3 pt[8] = {{-dxdzDz - dxdyDy1 - dx1, -dydzDz - dy1, -dz}, {-dxdzDz - dxdyDy1 + dx1, -dydzDz - dy1, -dz},
                        {-dxdzDz + dxdyDy1 - dx2, -dydzDz + dy1, -dz}, {-dxdzDz + dxdyDy1 + dx2, -dydzDz + dy1, -dz},
                        {+dxdzDz - dxdyDy2 - dx3, +dydzDz - dy2, +dz}, {+dxdzDz - dxdyDy2 + dx3, +dydzDz - dy2, +dz},
                        {+dxdzDz + dxdyDy2 - dx4, +dydzDz + dy2, +dz}, {+dxdzDz + dxdyDy2 + dx4, +dydzDz + dy2, +dz}};
    // plane through p1..p4 (clockwise seen from inside): n = (p3 - p1) x (p4 - p2) normalised
    // by multiplying with 1/|n|, d = -n . centroid
    auto plane = [&](int i, const Vec3 &p1, const Vec3 &p2, const Vec3 &p3, const Vec3 &p4) {
      const Vec3 a{p3.x - p1.x, p3.y - p1.y, p3.z - p1.z}, b{p4.x - p2.x, p4.y - p2.y, p4.z - p2.z};
      Vec3 n{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
      const double inv = 1. / std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
      n                = {n.x * inv, n.y * inv, n.z * inv};
      const Vec3 s{((p1.x + p2.x) + p3.x) + p4.x, ((p1.y + p2.y) + p3.y) + p4.y, ((p1.z + p2.z) + p3.z) + p4.z};
      const Vec3 c{0.25 * s.x, 0.25 * s.y, 0.25 * s.z};
      r[row::TrapA + i] = n.x;
      r[row::TrapB + i] = n.y;
      r[row::TrapC + i] = n.z;
      r[row::TrapD + i] = -(n.x * c.x + n.y * c.y + n.z * c.z);
    };
    plane(0, pt[0], pt[1], pt[5], pt[4]);  // ~ -Y
    plane(1, pt[2], pt[6], pt[7], pt[3]);  // ~ +Y
    plane(2, pt[0], pt[4], pt[6], pt[2]);  // ~ -X
    plane(3, pt[1], pt[3], pt[7], pt[5]);  // ~ +X
    r[row::TrapDz]         = dz;
    r[row::TrapTheta]      = theta;
    r[row::TrapPhi]        = phi;
    r[row::TrapDy1]        = dy1;
    r[row::TrapDx1]        = dx1;
    r[row::TrapDx2]        = dx2;
    r[row::TrapTanAlpha1]  = tanA1;
    r[row::TrapDy2]        = dy2;
    r[row::TrapDx3]        = dx3;
    r[row::TrapDx4]        = dx4;
    r[row::TrapTanAlpha2]  = tanA2;
    r[row::TrapTthetaCphi] = tcp;
    r[row::TrapTthetaSphi] = tsp;
    shape.insert(shape.end(), r, r + row::kTrapSize);
    return VGN_OK;
  }
  case kSphere: {
    // SphereStruct(rmin, rmax, sphi, dphi, stheta, dtheta) (SphereStruct.h:285-304):
    // CheckPhiAngles / CheckThetaAngles (SphereStruct.h:87-185) give the checked angles
    // and the full-range flags; the Wedge (source/Wedge_Evolution.cpp:17-99) and the
    // ThetaCone (ThetaCone_Evolution.h:62-82) keep the raw constructor angles.  Arguments
    // the reference only reports are rejected.
    const double rmin = p[0], rmax = p[1], sphi = p[2], dphi = p[3], stheta = p[4], dtheta = p[5];
    if (!(rmin >= 0 && rmax > rmin) || !(dphi > 0) || !(stheta >= 0 && stheta <= kPi) || !(dtheta > 0)) {
      err = "Sphere needs 0 <= rmin < rmax, dphi > 0, 0 <= stheta <= pi and dtheta > 0";
      return VGN_ERR_ARG;
    }
    const bool fullPhi     = dphi >= 2 * kPi - kAngTolerance * 0.5;
    const double dPhiChk   = fullPhi ? 2 * kPi : dphi;
    const double dThetaChk = dtheta + stheta >= kPi ? kPi - stheta : dtheta;
    const bool fullTheta   = !(dThetaChk - stheta < kPi);
    double sPhiChk         = 0;
    if (!fullPhi) {
      sPhiChk = sphi < 0 ? 2 * kPi - std::fmod(std::fabs(sphi), 2 * kPi) : std::fmod(sphi, 2 * kPi);
      if (sPhiChk + dPhiChk > 2 * kPi) sPhiChk -= 2 * kPi;
    }
    double r[row::kSphereSize] = {};
    r[row::SphRmin] = rmin;
    r[row::SphRmax] = rmax;
    wedge_fill(r + row::SphA1x, dphi, sphi);  // SphA1x..SphWedgeDPhi is a Wedge block
    const double sT = stheta, eT = stheta + dtheta;
    const double ts = sT > kPi / 2 ? kPi - sT : sT, te = eT > kPi / 2 ? kPi - eT : eT;
    r[row::SphSTheta]      = sT;
    r[row::SphETheta]      = eT;
    r[row::SphTanSTheta]   = std::tan(ts);
    r[row::SphTanETheta]   = std::tan(te);
    r[row::SphTanSTheta2]  = r[row::SphTanSTheta] * r[row::SphTanSTheta];
    r[row::SphTanETheta2]  = r[row::SphTanETheta] * r[row::SphTanETheta];
    r[row::SphTanBisector] = (sT > kPi / 2 && eT > kPi / 2) ? std::tan(ts - (dtheta / 2)) : std::tan(ts + (dtheta / 2));
    r[row::SphSlope1]      = std::tan(kPi / 2 - sT);
    r[row::SphSlope2]      = std::tan(kPi / 2 - eT);
    r[row::SphDPhi]        = dPhiChk;
    r[row::SphDTheta]      = dThetaChk;
    r[row::SphEThetaChk]   = stheta + dThetaChk;
    r[row::SphFullPhi]     = fullPhi ? 1. : 0.;
    r[row::SphFullTheta]   = fullTheta ? 1. : 0.;
    r[row::SphFull]        = fullPhi && fullTheta ? 1. : 0.;
    r[row::SphSPhi]        = sPhiChk;
    shape.insert(shape.end(), r, r + row::kSphereSize);
    return VGN_OK;
  }
  case kPolycone: {
    // UnplacedPolycone(phistart, deltaphi, Nz, z, rmin, rmax) -> PolyconeStruct::Init
    // (UnplacedPolycone.h:78-88, PolyconeStruct.h:144-291): planes reversed when z runs
    // downwards; a section (a ConeStruct built with the raw phi arguments) for every z
    // step larger than kTolerance, shifted to the step's centre.  rmin > rmax and a z
    // direction change, which the reference only reports, are rejected.
    const double sphi = p[0], dphi = p[1];
    const int nz      = (int)p[2];
    std::vector<double> z(nz), rin(nz), rout(nz);
    const bool rev = p[3] > p[3 + nz - 1];
    for (int i = 0; i < nz; ++i) {
      const int k = rev ? nz - 1 - i : i;
      z[i]        = p[3 + k];
      rin[i]      = p[3 + nz + k];
      rout[i]     = p[3 + 2 * nz + k];
    }
    for (int i = 0; i < nz; ++i)
      if (!(rin[i] >= 0 && rout[i] >= rin[i]) || (i > 0 && !(z[i] >= z[i - 1]))) {
        err = "Polycone needs 0 <= rmin <= rmax and monotonic z planes";
        return VGN_ERR_ARG;
      }
    std::vector<double> zs{z[0]}, shift, cones;
    double prevZ = z[0], prevRmin = rin[0], prevRmax = rout[0];
    const int dirZ = z[1] < z[0] ? -1 : 1;
    for (int i = 1; i < nz; ++i) {
      if (((z[i] > prevZ + kTolerance) && (dirZ > 0)) || ((z[i] < prevZ - kTolerance) && (dirZ < 0))) {
        const double cpar[7] = {prevRmin, prevRmax, rin[i], rout[i], (z[i] - prevZ) / 2, sphi, dphi};
        const int rc         = shape_make_row(kCone, cpar, 7, cones, err);
        if (rc) return rc;
        zs.push_back(z[i]);
        const size_t zi = zs.size() - 1;
        shift.push_back(zs[zi - 1] + 0.5 * (zs[zi] - zs[zi - 1]));
      }
      prevZ    = z[i];
      prevRmin = rin[i];
      prevRmax = rout[i];
    }
    const int nsec = (int)shift.size();
    if (nsec == 0) {
      err = "Polycone has no section longer than kTolerance";
      return VGN_ERR_ARG;
    }
    shape.push_back((double)nsec);
    shape.insert(shape.end(), zs.begin(), zs.end());
    shape.insert(shape.end(), shift.begin(), shift.end());
    shape.insert(shape.end(), cones.begin(), cones.end());
    shape.push_back(sphi);  // raw phi arguments, for the Extent (row::pcon_phi)
    shape.push_back(dphi);
    return VGN_OK;
  }
  case kPolyhedron: return polyhedron_row(p, shape, err);
  case kTorus: {
    // TorusStruct2(rmin, rmax, rtor, sphi, dphi) (TorusStruct2.h:36-43): the raw angles, the
    // squares, fPhiWedge(dphi, sphi) and the bounding GenericUnplacedTube(rtor - rmax - tol,
    // rtor + rmax + tol, rmax, sphi, dphi)
    if (!(p[0] >= 0 && p[1] > p[0] && p[2] > p[1] + kTolerance && p[4] > 0)) {
      err = "torus needs 0 <= rmin < rmax < rtor and dphi > 0";
      return VGN_ERR_ARG;
    }
    double r[row::kTorusSize];
    for (int k = 0; k < 5; ++k) r[row::TorRmin + k] = p[k];
    r[row::TorRmin2] = p[0] * p[0];
    r[row::TorRmax2] = p[1] * p[1];
    r[row::TorRtor2] = p[2] * p[2];
    wedge_fill(r + row::TorWedge, p[4], p[3]);
    const double tp[5] = {p[2] - p[1] - kTolerance, p[2] + p[1] + kTolerance, p[1], p[3], p[4]};
    std::vector<double> tube;
    if (int rc = shape_make_row(kTube, tp, 5, tube, err)) return rc;
    std::copy(tube.begin(), tube.end(), r + row::TorTube);
    shape.insert(shape.end(), r, r + row::kTorusSize);
    return VGN_OK;
  }
  case kCutTube: {
    // UnplacedCutTube(rmin, rmax, z, sphi, dphi, bx, by, bz, tx, ty, tz) -> CutTubeStruct
    // (UnplacedCutTube.h:54-70, CutTubeStruct.h:34-46): a tube of infinite half-length, the two
    // cut planes through (0, 0, -+z) with the normals made unit (Vector3D::Unit), then
    // Plane::Set (Plane.h:44-51: FixZeroes, 1 / Mag)
    if (!(p[7] < 0 && p[10] > 0)) {
      err = "cut tube needs a bottom normal with z < 0 and a top normal with z > 0";
      return VGN_ERR_ARG;
    }
    if (!(p[2] > 0)) {
      err = "cut tube needs dz > 0";
      return VGN_ERR_ARG;
    }
    const double tp[5] = {p[0], p[1], 1.7976931348623157e308, p[3], p[4]};  // kInfLength
    std::vector<double> tube;
    const int rc = shape_make_row(kTube, tp, 5, tube, err);
    if (rc) return rc;
    double r[row::kCutTubeSize];
    std::copy(tube.begin(), tube.end(), r);
    r[row::CutTubeDz] = p[2];
    for (int k = 0; k < 2; ++k) {
      const double *n0 = p + 5 + 3 * k;
      const double m   = std::sqrt((n0[0] * n0[0] + n0[1] * n0[1] + n0[2] * n0[2]) + 2.2250738585072014e-308);
      double f[3]      = {n0[0] / m, n0[1] / m, n0[2] / m};  // Vector3D::Unit (Vector3D.h:284-290)
      for (int i = 0; i < 3; ++i)
        if (std::fabs(f[i]) < kTolerance) f[i] = 0.0;
      const double inv = 1. / std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
      const double oz  = k == 0 ? -p[2] : p[2];
      double *n        = r + (k == 0 ? row::CutTubeN0 : row::CutTubeN1);
      for (int i = 0; i < 3; ++i) n[i] = inv * f[i];
      r[k == 0 ? row::CutTubeD0 : row::CutTubeD1] = inv * -(f[0] * 0. + f[1] * 0. + f[2] * oz);
    }
    r[row::CutTubeCos1]   = std::cos(p[3]);
    r[row::CutTubeSin1]   = std::sin(p[3]);
    r[row::CutTubeCos2]   = std::cos(p[3] + p[4]);
    r[row::CutTubeSin2]   = std::sin(p[3] + p[4]);
    r[row::CutTubeMaxVal] = p[1] > p[2] ? p[1] : p[2];
    shape.insert(shape.end(), r, r + row::kCutTubeSize);
    return VGN_OK;
  }
  case kOrb: {
    // OrbStruct fR (OrbStruct.h:19-25)
    if (!(p[0] > 0)) {
      err = "orb radius must be positive";
      return VGN_ERR_ARG;
    }
    shape.push_back(p[0]);
    return VGN_OK;
  }
  case kBoolean: {  // operands resolved by link_booleans (host_geometry.cpp) once placements are read
    auto is_id = [](double v) { return v >= 0. && v <= 2147483647. && v == std::floor(v); };
    if (!(p[0] == 0. || p[0] == 1. || p[0] == 2.) || !is_id(p[1]) || !is_id(p[2])) {
      err = "boolean: the operation must be 0, 1 or 2 and the operands placement ids";
      return VGN_ERR_ARG;
    }
    std::vector<double> b(row::kBoolSize, 0.);
    b[row::BoolOp]       = p[0];
    b[row::BoolLeftRow]  = p[1];  // operand placement ids until linked
    b[row::BoolRightRow] = p[2];
    b[row::BoolLeftType] = b[row::BoolRightType] = -1.;
    shape.insert(shape.end(), b.begin(), b.end());
    return VGN_OK;
  }
  default: err = "unsupported shape type " + std::to_string(type); return VGN_ERR_UNSUPPORTED;
  }
}

bool shape_row_has_sections(int32_t type, const double *r)
{
  switch (type) {
  case kTube:
  case kCutTube: return r[row::TubeDphi] < 2. * kPi;  // a cut tube's row starts with its tube's
  case kCone: return r[row::ConeDPhi] < 2. * kPi;
  case kPolycone: {  // the polycone's phi range lives in its section cones
    const int n = (int)r[row::PconNSec];
    return r[row::pcon_cone(n, 0) + row::ConeDPhi] < 2. * kPi;
  }
  case kSphere: return r[row::SphFull] == 0.;
  case kPolyhedron:
  case kTorus: return true;  // their kernels live in the sections set only
  case kBoolean:  // the operands' (once linked)
    return (r[row::BoolLeftType] >= 0 && shape_row_has_sections((int32_t)r[row::BoolLeftType], r + (int64_t)r[row::BoolLeftRow])) ||
           (r[row::BoolRightType] >= 0 && shape_row_has_sections((int32_t)r[row::BoolRightType], r + (int64_t)r[row::BoolRightRow]));
  default: return false;
  }
}

static inline double vmin(double a, double b) { return a < b ? a : b; }  // vecCore::math::Min
static inline double vmax(double a, double b) { return a > b ? a : b; }  // vecCore::math::Max

// VPlacedVolume::Extent (source/PlacedVolume.cpp:139-175) of a boolean's operand: its shape's
// extent taken into the boolean's frame (the eight corners when the placement rotates, else
// the two extremes)
static void operand_placed_extent(const double *b, int k, Vec3 &mn, Vec3 &mx)
{
  const int32_t type  = (int32_t)b[k == 0 ? row::BoolLeftType : row::BoolRightType];
  const double *orow  = b + (int64_t)b[k == 0 ? row::BoolLeftRow : row::BoolRightRow];
  const HostXForm x   = xform_from12(b + (k == 0 ? row::BoolLeftXf : row::BoolRightXf));
  Vec3 pmin, pmax;
  shape_extent(type, orow, pmin, pmax);
  if (x.has_rot) {
    const Vec3 c[8] = {{pmin.x, pmin.y, pmin.z}, {pmax.x, pmin.y, pmin.z}, {pmin.x, pmax.y, pmin.z},
                       {pmax.x, pmax.y, pmin.z}, {pmin.x, pmin.y, pmax.z}, {pmax.x, pmin.y, pmax.z},
                       {pmin.x, pmax.y, pmax.z}, {pmax.x, pmax.y, pmax.z}};
    mn = mx = xform_inverse_transform(x, c[0]);
    for (int i = 1; i < 8; ++i) {
      const Vec3 t = xform_inverse_transform(x, c[i]);
      mn           = {vmin(mn.x, t.x), vmin(mn.y, t.y), vmin(mn.z, t.z)};
      mx           = {vmax(mx.x, t.x), vmax(mx.y, t.y), vmax(mx.z, t.z)};
    }
  } else {
    mn = xform_inverse_transform(x, pmin);
    mx = xform_inverse_transform(x, pmax);
  }
}

// TransformedExtent (source/UnplacedBooleanVolume.cpp:403-442): the box of the operand's placed
// extent, whose corners it takes through the placement once more (the placed extent is already
// in the boolean's frame, so a moved operand's box comes out larger than the operand: the
// reference's extents, and so its bounding boxes, are these)
static void operand_transformed_extent(const double *b, int k, Vec3 &mn, Vec3 &mx)
{
  const HostXForm x = xform_from12(b + (k == 0 ? row::BoolLeftXf : row::BoolRightXf));
  Vec3 lower, upper;
  operand_placed_extent(b, k, lower, upper);
  const Vec3 delta{upper.x - lower.x, upper.y - lower.y, upper.z - lower.z};
  double minx = 1.7976931348623157e308, miny = minx, minz = minx;
  double maxx = -minx, maxy = -minx, maxz = -minx;
  for (int i = 0; i <= 1; ++i)
    for (int j = 0; j <= 1; ++j)
      for (int l = 0; l <= 1; ++l) {
        const Vec3 t = xform_inverse_transform(x, {lower.x + i * delta.x, lower.y + j * delta.y, lower.z + l * delta.z});
        minx = std::min(minx, t.x);
        miny = std::min(miny, t.y);
        minz = std::min(minz, t.z);
        maxx = std::max(maxx, t.x);
        maxy = std::max(maxy, t.y);
        maxz = std::max(maxz, t.z);
      }
  mn = {minx, miny, minz};
  mx = {maxx, maxy, maxz};
}

// UnplacedBooleanVolume<op>::Extent (source/UnplacedBooleanVolume.cpp:444-490)
static void boolean_extent(const double *b, Vec3 &mn, Vec3 &mx)
{
  Vec3 minL, maxL, minR, maxR;
  operand_transformed_extent(b, 0, minL, maxL);
  operand_transformed_extent(b, 1, minR, maxR);
  const int op = (int)b[row::BoolOp];
  if (op == 2) {
    mn = minL;
    mx = maxL;
  } else if (op == 0) {
    mn = {vmin(minL.x, minR.x), vmin(minL.y, minR.y), vmin(minL.z, minR.z)};
    mx = {vmax(maxL.x, maxR.x), vmax(maxL.y, maxR.y), vmax(maxL.z, maxR.z)};
  } else {
    mn = {vmax(minL.x, minR.x), vmax(minL.y, minR.y), vmax(minL.z, minR.z)};
    mx = {vmin(maxL.x, maxR.x), vmin(maxL.y, maxR.y), vmin(maxL.z, maxR.z)};
  }
}

void shape_extent(int32_t type, const double *r, Vec3 &mn, Vec3 &mx)
{
  switch (type) {
  case kBox:  // UnplacedBox::Extent (UnplacedBox.h:75-80)
    mn = {-r[0], -r[1], -r[2]};
    mx = {r[0], r[1], r[2]};
    return;
  case kTube: {  // UnplacedTube::Extent (source/UnplacedTube.cpp:214-266)
    const double rmax = r[row::TubeRmax], rmin = r[row::TubeRmin], sphi = r[row::TubeSphi], dphi = r[row::TubeDphi];
    const double *w = r + row::TubeWedge;
    mn = {-rmax, -rmax, -r[row::TubeZ]};
    mx = {rmax, rmax, r[row::TubeZ]};
    if (dphi == kTwoPi) return;
    const double Rin     = 0.5 * (rmax + rmin);
    const bool phi0out   = !wedge_contains(w, Rin, 0);
    const bool phi90out  = !wedge_contains(w, 0, Rin);
    const bool phi180out = !wedge_contains(w, -Rin, 0);
    const bool phi270out = !wedge_contains(w, 0, -Rin);
    if (!(phi0out || phi90out || phi180out || phi270out)) return;
    auto vmax = [](double a, double b) { return a > b ? a : b; };
    auto vmin = [](double a, double b) { return a < b ? a : b; };
    const double Cx = rmax * std::cos(sphi), Dx = rmax * std::cos(sphi + dphi);
    const double Cy = rmax * std::sin(sphi), Dy = rmax * std::sin(sphi + dphi);
    if (phi0out) mx.x = vmax(Cx, Dx);
    if (phi90out) mx.y = vmax(Cy, Dy);
    if (phi180out) mn.x = vmin(Cx, Dx);
    if (phi270out) mn.y = vmin(Cy, Dy);
    if (dphi >= kPi) return;
    const double Ax = rmin * std::cos(sphi), Bx = rmin * std::cos(sphi + dphi);
    const double Ay = rmin * std::sin(sphi), By = rmin * std::sin(sphi + dphi);
    double temp;
    temp = vmax(Ax, Bx);
    mx.x = temp > mx.x ? temp : mx.x;
    temp = vmax(Ay, By);
    mx.y = temp > mx.y ? temp : mx.y;
    temp = vmin(Ax, Bx);
    mn.x = temp < mn.x ? temp : mn.x;
    temp = vmin(Ay, By);
    mn.y = temp < mn.y ? temp : mn.y;
    return;
  }
  case kCone: {  // UnplacedCone::Extent (source/UnplacedCone.cpp:146-206, the phi-aware definition)
    const double max = r[row::ConeArgRmax1] > r[row::ConeArgRmax2] ? r[row::ConeArgRmax1] : r[row::ConeArgRmax2];
    const double min = r[row::ConeArgRmin1] > r[row::ConeArgRmin2] ? r[row::ConeArgRmin2] : r[row::ConeArgRmin1];
    const double sphi = r[row::ConeSPhi], dphi = r[row::ConeDPhi];
    const double *w = r + row::ConeWedge;
    mn = {-max, -max, -r[row::ConeDz]};
    mx = {max, max, r[row::ConeDz]};
    if (dphi == kTwoPi) return;
    const double Rin     = 0.5 * (max + min);
    const bool phi0out   = !wedge_contains(w, Rin, 0);
    const bool phi90out  = !wedge_contains(w, 0, Rin);
    const bool phi180out = !wedge_contains(w, -Rin, 0);
    const bool phi270out = !wedge_contains(w, 0, -Rin);
    if (!(phi0out || phi90out || phi180out || phi270out)) return;
    auto vmax = [](double a, double b) { return a > b ? a : b; };
    auto vmin = [](double a, double b) { return a < b ? a : b; };
    const double Cx = max * std::cos(sphi), Dx = max * std::cos(sphi + dphi);
    const double Cy = max * std::sin(sphi), Dy = max * std::sin(sphi + dphi);
    if (phi0out) mx.x = vmax(Cx, Dx);
    if (phi90out) mx.y = vmax(Cy, Dy);
    if (phi180out) mn.x = vmin(Cx, Dx);
    if (phi270out) mn.y = vmin(Cy, Dy);
    if (dphi >= kPi) return;
    const double Ax = min * std::cos(sphi), Bx = min * std::cos(sphi + dphi);
    const double Ay = min * std::sin(sphi), By = min * std::sin(sphi + dphi);
    double temp;
    temp = vmax(Ax, Bx);
    mx.x = temp > mx.x ? temp : mx.x;
    temp = vmax(Ay, By);
    mx.y = temp > mx.y ? temp : mx.y;
    temp = vmin(Ax, Bx);
    mn.x = temp < mn.x ? temp : mn.x;
    temp = vmin(Ay, By);
    mn.y = temp < mn.y ? temp : mn.y;
    return;
  }
  case kTrd: {  // UnplacedTrd::Extent (UnplacedTrd.h:218-222)
    const double mxx = r[row::TrdDx1] > r[row::TrdDx2] ? r[row::TrdDx1] : r[row::TrdDx2];
    const double mxy = r[row::TrdDy1] > r[row::TrdDy2] ? r[row::TrdDy1] : r[row::TrdDy2];
    mn = {-mxx, -mxy, -r[row::TrdDz]};
    mx = {mxx, mxy, r[row::TrdDz]};
    return;
  }
  case kTrapezoid: {  // UnplacedTrapezoid::Extent through fromPlanesToCorners (source/UnplacedTrapezoid.cpp:297-337, 467-494)
    const double dz = r[row::TrapDz];
    const double *A = r + row::TrapA, *B = r + row::TrapB, *C = r + row::TrapC, *D = r + row::TrapD;
    double y[8], x[8];
    y[0] = y[1] = -(D[0] - dz * C[0]) / B[0];
    y[2] = y[3] = -(D[1] - dz * C[1]) / B[1];
    y[4] = y[5] = -(D[0] + dz * C[0]) / B[0];
    y[6] = y[7] = -(D[1] + dz * C[1]) / B[1];
    x[0] = ((B[2] / B[0]) * (D[0] - dz * C[0]) - (D[2] - dz * C[2])) / A[2];
    x[1] = ((B[3] / B[0]) * (D[0] - dz * C[0]) - (D[3] - dz * C[3])) / A[3];
    x[2] = ((B[2] / B[1]) * (D[1] - dz * C[1]) - (D[2] - dz * C[2])) / A[2];
    x[3] = ((B[3] / B[1]) * (D[1] - dz * C[1]) - (D[3] - dz * C[3])) / A[3];
    x[4] = ((B[2] / B[0]) * (D[0] + dz * C[0]) - (D[2] + dz * C[2])) / A[2];
    x[5] = ((B[3] / B[0]) * (D[0] + dz * C[0]) - (D[3] + dz * C[3])) / A[3];
    x[6] = ((B[2] / B[1]) * (D[1] + dz * C[1]) - (D[2] + dz * C[2])) / A[2];
    x[7] = ((B[3] / B[1]) * (D[1] + dz * C[1]) - (D[3] + dz * C[3])) / A[3];
    auto mx2 = [](double a, double b) { return a > b ? a : b; };
    auto mn2 = [](double a, double b) { return a < b ? a : b; };
    auto tree = [](const double *v, auto f) { return f(f(f(v[0], v[1]), f(v[2], v[3])), f(f(v[4], v[5]), f(v[6], v[7]))); };
    mn = {tree(x, mn2), tree(y, mn2), -dz};
    mx = {tree(x, mx2), tree(y, mx2), dz};
    return;
  }
  case kSphere: {  // UnplacedSphere::Extent with the phi and theta cuts (source/UnplacedSphere.cpp:74-158)
    auto vmin = [](double a, double b) { return a < b ? a : b; };
    auto vmax = [](double a, double b) { return a > b ? a : b; };
    const double rmax = r[row::SphRmax], rmin = r[row::SphRmin];
    const double sTheta = r[row::SphSTheta], eTheta = r[row::SphEThetaChk];
    mn = {-rmax, -rmax, -rmax};
    mx = {rmax, rmax, rmax};
    if (r[row::SphFull] != 0.) return;
    double st1 = 0., st2 = 0.;
    if (r[row::SphFullTheta] == 0.) {
      mx.z = ((sTheta <= kPi / 2.) ? rmax : rmin) * std::cos(sTheta);
      mn.z = ((eTheta <= kPi / 2.) ? rmin : rmax) * std::cos(eTheta);
      st1  = std::sin(sTheta);
      st2  = std::sin(eTheta);
      if (sTheta <= kPi / 2.) {
        if (eTheta < kPi / 2.) {
          mx.x = rmax * st2;
          mn.x = -rmax * st2;
          mx.y = rmax * st2;
          mn.y = -rmax * st2;
        }
      } else {
        mx.x = rmax * st1;
        mn.x = -rmax * st1;
        mx.y = rmax * st1;
        mn.y = -rmax * st1;
      }
    }
    if (r[row::SphFullPhi] == 0.) {
      double Rmax = rmax;
      if (sTheta > kPi / 2.) Rmax *= st1;
      if (eTheta < kPi / 2.) Rmax *= st2;
      const double Rmin = rmin * vmin(st1, st2);
      const double Rin  = 0.5 * (Rmax + Rmin);
      const double *w   = r + row::SphA1x;
      const bool phi0out   = !wedge_contains(w, Rin, 0);
      const bool phi90out  = !wedge_contains(w, 0, Rin);
      const bool phi180out = !wedge_contains(w, -Rin, 0);
      const bool phi270out = !wedge_contains(w, 0, -Rin);
      if (!(phi0out || phi90out || phi180out || phi270out)) return;
      const double sphi = r[row::SphSPhi], dphi = r[row::SphDPhi];
      const double Cx = Rmax * std::cos(sphi), Dx = Rmax * std::cos(sphi + dphi);
      const double Cy = Rmax * std::sin(sphi), Dy = Rmax * std::sin(sphi + dphi);
      if (phi0out) mx.x = vmax(Cx, Dx);
      if (phi90out) mx.y = vmax(Cy, Dy);
      if (phi180out) mn.x = vmin(Cx, Dx);
      if (phi270out) mn.y = vmin(Cy, Dy);
      if (dphi >= kPi) return;
      const double Ax = Rmin * std::cos(sphi), Bx = Rmin * std::cos(sphi + dphi);
      const double Ay = Rmin * std::sin(sphi), By = Rmin * std::sin(sphi + dphi);
      double temp;
      temp = vmax(Ax, Bx);
      mx.x = temp > mx.x ? temp : mx.x;
      temp = vmax(Ay, By);
      mx.y = temp > mx.y ? temp : mx.y;
      temp = vmin(Ax, Bx);
      mn.x = temp < mn.x ? temp : mn.x;
      temp = vmin(Ay, By);
      mn.y = temp < mn.y ? temp : mn.y;
    }
    return;
  }
  case kPolycone: {
    // UnplacedPolycone::Extent (source/UnplacedPolycone.cpp:865-902): z from the end planes;
    // x and y from the Extent of Cone(minR, maxR, minR, maxR, 1, fStartPhi, fDeltaPhi), the
    // sections' smallest constructor rmin and largest rmax and the polycone's phi range
    // (PolyconeStruct::Init, PolyconeStruct.h:152-184)
    const int n = (int)r[row::PconNSec];
    auto vmax   = [](double a, double b) { return a > b ? a : b; };
    auto vmin   = [](double a, double b) { return a < b ? a : b; };
    double maxR = 0, minR = 1.7976931348623157e308;  // kInfLength
    for (int k = 0; k < n; ++k) {
      const double *c = r + row::pcon_cone(n, k);
      maxR            = vmax(maxR, vmax(c[row::ConeArgRmax1], c[row::ConeArgRmax2]));
      minR            = vmin(minR, vmin(c[row::ConeArgRmin1], c[row::ConeArgRmin2]));
    }
    const double phiStart = r[row::pcon_phi(n)], phiTotal = r[row::pcon_phi(n) + 1];
    double dphi = phiTotal >= kTwoPi - 0.5 * kAngTolerance ? kTwoPi : phiTotal;  // SetAndCheckDPhiAngle
    double sphi = 0;
    if (phiTotal <= 0. || phiTotal > kTwoPi - kTolerance) {
      dphi = kTwoPi;
    } else {
      sphi = phiStart;
      while (sphi < 0) sphi += kTwoPi;
    }
    std::vector<double> cone;
    std::string unused;
    const double cpar[7] = {minR, maxR, minR, maxR, 1, sphi, dphi};
    shape_make_row(kCone, cpar, 7, cone, unused);
    shape_extent(kCone, cone.data(), mn, mx);
    const double z0 = r[row::PconZs], zn = r[row::PconZs + n];
    mn.z = z0 > zn ? zn : z0;
    mx.z = z0 > zn ? z0 : zn;
    return;
  }
  case kCutTube: {  // UnplacedCutTube::Extent (source/UnplacedCutTube.cpp:128-172)
    const double rmax = r[row::TubeRmax], rmin = r[row::TubeRmin], sphi = r[row::TubeSphi], dphi = r[row::TubeDphi];
    const double *w = r + row::TubeWedge, *bn = r + row::CutTubeN0, *tn = r + row::CutTubeN1, z = r[row::CutTubeDz];
    auto vmax = [](double a, double b) { return a > b ? a : b; };
    auto vmin = [](double a, double b) { return a < b ? a : b; };
    auto zlim = [&](bool top, double rv, double ph) {  // ZlimitTop / ZlimitBottom (UnplacedCutTube.h:135-147)
      const double *n = top ? tn : bn;
      return (top ? z : -z) - (rv / n[2]) * (n[0] * std::cos(ph) + n[1] * std::sin(ph));
    };
    const double dztop    = rmax * std::sqrt(1. - tn[2] * tn[2]) / tn[2];
    const double dzbottom = -rmax * std::sqrt(1. - bn[2] * bn[2]) / bn[2];
    mn = {-rmax, -rmax, -z - dzbottom};
    mx = {rmax, rmax, z + dztop};
    if (dphi == kTwoPi) return;
    const double c1 = r[row::CutTubeCos1], s1 = r[row::CutTubeSin1], c2 = r[row::CutTubeCos2], s2 = r[row::CutTubeSin2];
    if (!wedge_contains(w, -tn[0], -tn[1])) {
      mx.z = vmax(zlim(true, rmax, sphi), zlim(true, rmax, sphi + dphi));
      mx.z = vmax(mx.z, vmax(zlim(true, rmin, sphi), zlim(true, rmin, sphi + dphi)));
    }
    if (!wedge_contains(w, -bn[0], -bn[1])) {
      mn.z = vmin(zlim(false, rmax, sphi), zlim(false, rmax, sphi + dphi));
      mn.z = vmin(mn.z, vmin(zlim(false, rmin, sphi), zlim(false, rmin, sphi + dphi)));
    }
    if (!wedge_contains(w, 1., 0.)) {
      mx.x = vmax(rmax * c1, rmax * c2);
      mx.x = vmax(mx.x, vmax(rmin * c1, rmin * c2));
    }
    if (!wedge_contains(w, -1., 0.)) {
      mn.x = vmin(rmax * c1, rmax * c2);
      mn.x = vmin(mn.x, vmin(rmin * c1, rmin * c2));
    }
    if (!wedge_contains(w, 0., 1.)) {
      mx.y = vmax(rmax * s1, rmax * s2);
      mx.y = vmax(mx.y, vmax(rmin * s1, rmin * s2));
    }
    if (!wedge_contains(w, 0., -1.)) {
      mn.y = vmin(rmax * s1, rmax * s2);
      mn.y = vmin(mn.y, vmin(rmin * s1, rmin * s2));
    }
    return;
  }
  case kOrb:  // UnplacedOrb::Extent (source/UnplacedOrb.cpp:58-63)
    mn = {-r[0], -r[0], -r[0]};
    mx = {r[0], r[0], r[0]};
    return;
  case kBoolean: boolean_extent(r, mn, mx); return;
  case kTorus: shape_extent(kTube, r + row::TorTube, mn, mx); return;  // UnplacedTorus2.h:210
  case kPolyhedron: {  // UnplacedPolyhedron::Extent (source/UnplacedPolyhedron.cpp:273-303)
    const int S = (int)r[row::PhdSides], nz = (int)r[row::PhdNz];
    const double sidePhi = r[row::PhdPhiDelta] / S, conv = 1. / std::cos(0.5 * sidePhi);
    double a[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, b[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int iphi = 0; iphi <= S; ++iphi) {
      const double phi = r[row::PhdPhiStart] + iphi * sidePhi;
      const double cx = conv * std::cos(phi), cy = conv * std::sin(phi);
      for (int iz = 0; iz < nz; ++iz)
        for (int w = 0; w < 2; ++w) {
          const double rr   = r[(w == 0 ? row::phd_rmin(nz) : row::phd_rmax(nz)) + iz];
          const double c[3] = {rr * cx, rr * cy, r[row::phd_z(nz) + iz]};
          for (int k = 0; k < 3; ++k) {
            a[k] = vmin(a[k], c[k]);
            b[k] = vmax(b[k], c[k]);
          }
        }
    }
    mn = {a[0], a[1], a[2]};
    mx = {b[0], b[1], b[2]};
    return;
  }
  default: mn = mx = {0, 0, 0};
  }
}

}  // namespace vgn
