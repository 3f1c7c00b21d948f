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

int shape_param_count(int32_t type, const double *p, int32_t n_avail)
{
  (void)p;
  (void)n_avail;
  switch (type) {
  case kBox: return 3;
  case kTube: return 5;
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
  default: mn = mx = {0, 0, 0};
  }
}

}  // namespace vgn
