// host_shapes.cpp -- shape parameter rows and extents (host side).
//
// A row holds the shape's defining parameters plus the cached members the
// reference precomputes in its *Struct constructors, computed with the same
// expressions so the device kernels see the same doubles.
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

int shape_param_count(int32_t type, const double *p, int32_t n_avail)
{
  (void)p;
  (void)n_avail;
  switch (type) {
  case kBox: return 3;
  case kTube: return 5;
  case kCone: return 7;
  default: return -1;
  }
}

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
    // TubeStruct(rmin, rmax, z, sphi, dphi) + CalculateCached (TubeStruct.h:43-72, 153-175)
    const double rmin = p[0] < 0.0 ? 0.0 : p[0], rmax = p[1], z = p[2], dphi = p[4];
    if (dphi < kTwoPi) {
      err = "tube phi sections are not supported";
      return VGN_ERR_UNSUPPORTED;
    }
    if (!(rmax > rmin && z > 0)) {
      err = "tube needs rmax > rmin and dz > 0";
      return VGN_ERR_ARG;
    }
    double row[row::kTubeSize];
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
    if (p[6] < kTwoPi - 0.5 * kAngTolerance) {
      err = "cone phi sections are not supported";
      return VGN_ERR_UNSUPPORTED;
    }
    double rmin1 = p[0] < 0.0 ? 0.0 : p[0], rmax1 = p[1], rmin2 = p[2] < 0.0 ? 0.0 : p[2], rmax2 = p[3];
    const double dz = p[4];
    if (!(dz > 0 && rmax1 >= rmin1 && rmax2 >= rmin2 && (rmax1 > 0 || rmax2 > 0))) {
      err = "cone needs dz > 0 and rmax >= rmin at both ends";
      return VGN_ERR_ARG;
    }
    double r[row::kConeSize];
    r[row::ConeArgRmax1]  = p[1];
    r[row::ConeArgRmax2]  = p[3];
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
  default: err = "unsupported shape type " + std::to_string(type); return VGN_ERR_UNSUPPORTED;
  }
}

void shape_extent(int32_t type, const double *r, Vec3 &mn, Vec3 &mx)
{
  switch (type) {
  case kBox:  // UnplacedBox::Extent (UnplacedBox.h:75-80)
    mn = {-r[0], -r[1], -r[2]};
    mx = {r[0], r[1], r[2]};
    return;
  case kTube:  // UnplacedTube::Extent, full phi (source/UnplacedTube.cpp:214-220)
    mn = {-r[row::TubeRmax], -r[row::TubeRmax], -r[row::TubeZ]};
    mx = {r[row::TubeRmax], r[row::TubeRmax], r[row::TubeZ]};
    return;
  case kCone: {  // UnplacedCone::Extent, full phi (source/UnplacedCone.cpp:149-165)
    const double m = r[row::ConeArgRmax1] > r[row::ConeArgRmax2] ? r[row::ConeArgRmax1] : r[row::ConeArgRmax2];
    mn = {-m, -m, -r[row::ConeDz]};
    mx = {m, m, r[row::ConeDz]};
    return;
  }
  default: mn = mx = {0, 0, 0};
  }
}

}  // namespace vgn
