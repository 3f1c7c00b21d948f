// vgnav.hpp -- header-only C++ host interface over the libvgnav C ABI.
//
// Mirrors the batched part of VecGeom's navigator interface
// (VecGeom/navigation/VNavigator.h:878-975) for C++ callers: SOA3D views of
// points and directions, a pool of NavStateIndex-layout states, and a
// BVHNavigator whose methods keep the reference's names and argument order.
// Errors throw vgnav::Error (status code + message from vgn_last_error()).
#ifndef VGNAV_HPP
#define VGNAV_HPP

#include <cstddef>
#include <stdexcept>
#include <string>

#include "vgnav.h"

namespace vgnav {

class Error : public std::runtime_error {
public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

private:
  int code_;
};

inline void check(int rc)
{
  if (rc != VGN_OK) throw Error(rc, std::string("vgnav: ") + vgn_last_error());
}

// Non-owning SOA3D<double> view (VecGeom/base/SOA3D.h:179): three coordinate arrays.
struct SOA3D {
  const double *x, *y, *z;
  std::size_t n;
  std::size_t size() const { return n; }
};

// Mutable view on caller-owned states (NavStatePool / NavigationState** in the reference).
struct NavStatePool {
  vgn_state *states;
  std::size_t n;
  std::size_t size() const { return n; }
};

// A closed geometry resident on one GPU (replaces GeoManager::CloseGeometry +
// BVHManager::Init + CudaManager upload + BVHManager::DeviceInit).
class Geometry {
public:
  Geometry(const vgn_geometry_desc &desc, int device) { check(vgn_geometry_create(&desc, device, &g_)); }
  ~Geometry() { vgn_geometry_free(g_); }
  Geometry(const Geometry &)            = delete;
  Geometry &operator=(const Geometry &) = delete;
  const vgn_geometry *get() const { return g_; }
  std::size_t device_bytes() const
  {
    std::size_t b = 0;
    check(vgn_geometry_device_bytes(g_, &b));
    return b;
  }

private:
  vgn_geometry *g_ = nullptr;
};

// BVH navigator over a resident geometry; `flags` selects VGN_PRECISION_FP64
// (default) or VGN_PRECISION_MIXED.  Pointers may be host or device memory.
class BVHNavigator {
public:
  explicit BVHNavigator(const Geometry &geom, int flags = VGN_PRECISION_FP64, void *stream = nullptr)
      : g_(geom.get()), flags_(flags), stream_(stream)
  {
  }

  // VNavigator::ComputeStepsAndSafetiesAndPropagatedStates (VNavigator.h:913-941)
  void ComputeStepsAndSafetiesAndPropagatedStates(const SOA3D &globalpoints, const SOA3D &globaldirs,
                                                  const double *step_limit, const NavStatePool &in_states,
                                                  NavStatePool &out_states, double *out_steps,
                                                  double *out_safeties) const
  {
    check(vgn_compute_step_batch(g_, (int64_t)globalpoints.size(), globalpoints.x, globalpoints.y, globalpoints.z,
                                 globaldirs.x, globaldirs.y, globaldirs.z, step_limit, in_states.states,
                                 out_states.states, out_steps, out_safeties, flags_, stream_));
  }

  // VNavigator::ComputeStepsAndPropagatedStates (VNavigator.h:878-907)
  void ComputeStepsAndPropagatedStates(const SOA3D &globalpoints, const SOA3D &globaldirs, const double *step_limit,
                                       const NavStatePool &in_states, NavStatePool &out_states,
                                       double *out_steps) const
  {
    ComputeStepsAndSafetiesAndPropagatedStates(globalpoints, globaldirs, step_limit, in_states, out_states,
                                               out_steps, nullptr);
  }

  // ComputeStep (no relocation, VNavigator.h:494-540) over a batch
  void ComputeSteps(const SOA3D &globalpoints, const SOA3D &globaldirs, const double *step_limit,
                    const NavStatePool &in_states, NavStatePool &out_states, double *out_steps) const
  {
    check(vgn_compute_step_batch(g_, (int64_t)globalpoints.size(), globalpoints.x, globalpoints.y, globalpoints.z,
                                 globaldirs.x, globaldirs.y, globaldirs.z, step_limit, in_states.states,
                                 out_states.states, out_steps, nullptr, flags_ | VGN_NO_RELOCATE, stream_));
  }

  // VSafetyEstimatorHelper::ComputeSafety (VSafetyEstimator.h:98-107) over a batch
  void ComputeSafeties(const SOA3D &globalpoints, const NavStatePool &states, double *out_safeties) const
  {
    check(vgn_compute_safety_batch(g_, (int64_t)globalpoints.size(), globalpoints.x, globalpoints.y,
                                   globalpoints.z, states.states, out_safeties, flags_, stream_));
  }

  // GlobalLocator::LocateGlobalPoint(world, p, state, true) over a batch
  void LocatePoints(const SOA3D &globalpoints, NavStatePool &out_states) const
  {
    check(vgn_locate_batch(g_, (int64_t)globalpoints.size(), globalpoints.x, globalpoints.y, globalpoints.z,
                           out_states.states, flags_, stream_));
  }

  void Synchronize() const { check(vgn_synchronize(g_, stream_)); }

private:
  const vgn_geometry *g_;
  int flags_;
  void *stream_;
};

}  // namespace vgnav

#endif
