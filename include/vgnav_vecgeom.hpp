// vgnav_vecgeom.hpp -- drop-in GPU navigator for VecGeom 1.2.0 applications.
//
// Include this header in a program built against VecGeom (navigation-index build,
// VECGEOM_USE_NAVINDEX, which CUDA builds force; CMakeLists.txt:163-166) and link
// libvgnav.  It provides
//
//   vgnav::ExportGeometry()        the closed geometry of vecgeom::GeoManager as the
//                                  flat vgn_geometry_desc of vgnav.h (shapes with their
//                                  constructor parameters, placements in id order)
//   vgnav::GpuBVHNavigator         a vecgeom::VNavigator whose batch calls run on the GPU
//
// GpuBVHNavigator is a VNavigatorHelper (VecGeom/navigation/VNavigator.h:331-1097) with
// the hooks of BVHNavigator (BVHNavigator.h:35-61), so its scalar calls are VecGeom's
// own BVH navigation on the host, and it overrides the three batch virtuals
//   ComputeStepsAndPropagatedStates(SOA3D, SOA3D, Precision const*, NavigationState const* const*,
//                                   NavigationState**, Precision*)                 (VNavigator.h:878-907)
//   ComputeStepsAndSafetiesAndPropagatedStates(SOA3D, SOA3D, Precision const*, NavStatePool const&,
//                                   NavStatePool&, Precision*, bool const*, Precision*) (VNavigator.h:913-941)
//   ComputeStepsAndSafetiesAndPropagatedStates(..., NavigationState const* const*,
//                                   NavigationState**, ..., bool const*, Precision*)  (VNavigator.h:947-975)
// to call vgn_compute_step_batch.  A caller that already batches, such as
// test/benchmark/NavigationKernelBenchmarker.cpp:360-368, keeps its code:
//
//     vgnav::GpuBVHNavigator gpu(/*device=*/0);           // after GeoManager::CloseGeometry
//     for (auto &lv : GeoManager::Instance().GetLogicalVolumesMap())
//       if (lv.second->GetDaughters().size()) lv.second->SetNavigator(&gpu);
//     nav->ComputeStepsAndSafetiesAndPropagatedStates(points, dirs, slimits, *inpool, *outpool,
//                                                     steps, calcsafeties, safeties);
//
// Results equal VecGeom's BVHNavigator bit for bit (FP64 and mixed forms alike).
// Unlike the reference batch call, tracks of one batch may sit in different volumes.
// Arrays may be host memory (the usual SOA3D and NavStatePool; the library stages them)
// or device memory.  Errors throw vgnav::Error with the library's status and message.
//
// Boolean solids export as their operation and the ids of their placed operands, which
// keep VecGeom's ids and get the mother VGN_BOOLEAN_OPERAND.
//
// Shape parameters are exported as the shapes hold them.  They reproduce the shape exactly
// when the shape keeps its constructor's values: full-range shapes, and phi sections whose
// start angle lies in [0, 2 pi) and whose end does not pass 2 pi.  Trapezoids keep
// tan(alpha) only; the exporter recovers an alpha whose tangent is that value exactly.
#ifndef VGNAV_VECGEOM_HPP
#define VGNAV_VECGEOM_HPP

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "VecGeom/base/SOA3D.h"
#include "VecGeom/management/BVHManager.h"
#include "VecGeom/management/GeoManager.h"
#include "VecGeom/navigation/BVHSafetyEstimator.h"
#include "VecGeom/navigation/NavStatePool.h"
#include "VecGeom/navigation/NavigationState.h"
#include "VecGeom/navigation/VNavigator.h"
#include "VecGeom/volumes/LogicalVolume.h"
#include "VecGeom/volumes/PlacedVolume.h"
#include "VecGeom/volumes/UnplacedBooleanVolume.h"
#include "VecGeom/volumes/UnplacedBox.h"
#include "VecGeom/volumes/UnplacedCone.h"
#include "VecGeom/volumes/UnplacedCutTube.h"
#include "VecGeom/volumes/UnplacedOrb.h"
#include "VecGeom/volumes/UnplacedPolycone.h"
#include "VecGeom/volumes/UnplacedPolyhedron.h"
#include "VecGeom/volumes/UnplacedSphere.h"
#include "VecGeom/volumes/UnplacedTorus2.h"
#include "VecGeom/volumes/UnplacedTrapezoid.h"
#include "VecGeom/volumes/UnplacedTrd.h"
#include "VecGeom/volumes/UnplacedTube.h"
#include "vgnav.h"
#include "vgnav.hpp"

namespace vgnav {

static_assert(sizeof(vecgeom::NavigationState) == sizeof(vgn_state),
              "GpuBVHNavigator needs the 12-byte NavStateIndex states (VECGEOM_USE_NAVINDEX)");

// The flat description of a closed VecGeom geometry; desc() points into this object.
struct ExportedGeometry {
  std::vector<int32_t> lv_shape, lv_param_offset, pv_logical, pv_mother;
  std::vector<double> params, pv_transform;
  int32_t world_placed = -1;
  vgn_geometry_desc desc() const
  {
    return vgn_geometry_desc{(int32_t)lv_shape.size(), lv_shape.data(),       lv_param_offset.data(),
                             params.data(),            (int32_t)params.size(), (int32_t)pv_logical.size(),
                             pv_logical.data(),        pv_mother.data(),       pv_transform.data(),
                             world_placed};
  }
};

namespace detail {

// an alpha whose tangent is exactly t (the trapezoid keeps tan(alpha) only,
// TrapezoidStruct.h:47): atan(t), or one of its nearest neighbours
inline double alpha_with_tangent(double t)
{
  const double a0 = std::atan(t);
  double lo = a0, hi = a0;
  for (int k = 0; k < 8; ++k) {
    if (std::tan(lo) == t) return lo;
    if (std::tan(hi) == t) return hi;
    lo = std::nextafter(lo, -1e300);
    hi = std::nextafter(hi, 1e300);
  }
  return a0;
}

// shape type and parameter row of one unplaced volume (vgn_shape_type numbering); -1 if
// the shape has no kernel in libvgnav
inline int shape_row(vecgeom::VUnplacedVolume const *u, std::vector<double> &p)
{
  using namespace vecgeom;
  if (auto b = dynamic_cast<UnplacedBox const *>(u)) {
    p = {b->x(), b->y(), b->z()};
    return VGN_BOX;
  }
  if (auto t = dynamic_cast<UnplacedTube const *>(u)) {
    p = {t->rmin(), t->rmax(), t->z(), t->sphi(), t->dphi()};
    return VGN_TUBE;
  }
  if (auto c = dynamic_cast<UnplacedCone const *>(u)) {
    p = {c->GetRmin1(), c->GetRmax1(), c->GetRmin2(), c->GetRmax2(), c->GetDz(), c->GetSPhi(), c->GetDPhi()};
    return VGN_CONE;
  }
  if (auto d = dynamic_cast<UnplacedTrd const *>(u)) {
    p = {d->dx1(), d->dx2(), d->dy1(), d->dy2(), d->dz()};
    return VGN_TRD;
  }
  if (auto z = dynamic_cast<UnplacedTrapezoid const *>(u)) {
    auto const &s = z->GetStruct();
    p = {s.fDz,  s.fTheta, s.fPhi, s.fDy1, s.fDx1, s.fDx2, alpha_with_tangent(s.fTanAlpha1),
         s.fDy2, s.fDx3,   s.fDx4, alpha_with_tangent(s.fTanAlpha2)};
    return VGN_TRAPEZOID;
  }
  if (auto s = dynamic_cast<UnplacedSphere const *>(u)) {
    p = {s->GetInnerRadius(),     s->GetOuterRadius(),     s->GetStartPhiAngle(),
         s->GetDeltaPhiAngle(),   s->GetStartThetaAngle(), s->GetDeltaThetaAngle()};
    return VGN_SPHERE;
  }
  if (auto c = dynamic_cast<UnplacedCutTube const *>(u)) {  // the cut planes' unit normals
    const auto b = c->BottomNormal(), t = c->TopNormal();
    p = {c->rmin(), c->rmax(), c->z(), c->sphi(), c->dphi(), b.x(), b.y(), b.z(), t.x(), t.y(), t.z()};
    return VGN_CUTTUBE;
  }
  if (auto o = dynamic_cast<UnplacedOrb const *>(u)) {
    p = {o->GetRadius()};
    return VGN_ORB;
  }
  // booleans: the operation and the ids of the two placed operands (BooleanStruct.h:23-25)
  BooleanStruct const *bs = nullptr;
  if (auto b = dynamic_cast<UnplacedBooleanVolume<kUnion> const *>(u)) bs = &b->GetStruct();
  if (auto b = dynamic_cast<UnplacedBooleanVolume<kIntersection> const *>(u)) bs = &b->GetStruct();
  if (auto b = dynamic_cast<UnplacedBooleanVolume<kSubtraction> const *>(u)) bs = &b->GetStruct();
  if (bs) {
    const int op = bs->fOp == kUnion ? VGN_BOOL_UNION : bs->fOp == kIntersection ? VGN_BOOL_INTERSECTION
                                                                                  : VGN_BOOL_SUBTRACTION;
    p = {(double)op, (double)bs->fLeftVolume->id(), (double)bs->fRightVolume->id()};
    return VGN_BOOLEAN;
  }
  if (auto t = dynamic_cast<UnplacedTorus2 const *>(u)) {
    p = {t->rmin(), t->rmax(), t->rtor(), t->sphi(), t->dphi()};
    return VGN_TORUS2;
  }
  if (auto h = dynamic_cast<UnplacedPolyhedron const *>(u)) {  // the planes the struct keeps
    const int nz = (int)h->GetZPlanes().size();
    p            = {h->GetPhiStart(), h->GetPhiDelta(), (double)h->GetSideCount(), (double)nz};
    for (int i = 0; i < nz; ++i) p.push_back(h->GetZPlanes()[i]);
    for (int i = 0; i < nz; ++i) p.push_back(h->GetRMin()[i]);
    for (int i = 0; i < nz; ++i) p.push_back(h->GetRMax()[i]);
    return VGN_POLYHEDRON;
  }
  if (auto c = dynamic_cast<UnplacedPolycone const *>(u)) {
    auto const *h = c->GetOriginalParameters();  // the constructor's planes (PolyconeStruct.h:279-285)
    if (!h) return -1;
    const int nz = h->fHNum_z_planes;
    p        = {h->fHStart_angle, h->fHOpening_angle, (double)nz};
    for (int i = 0; i < nz; ++i) p.push_back(h->fHZ_values[i]);
    for (int i = 0; i < nz; ++i) p.push_back(h->fHRmin[i]);
    for (int i = 0; i < nz; ++i) p.push_back(h->fHRmax[i]);
    return VGN_POLYCONE;
  }
  return -1;
}

} // namespace detail

// The geometry closed by vecgeom::GeoManager, described for vgn_geometry_create:
// logical volumes by id with their shapes, placed volumes by id with the logical
// volume they place, the logical volume whose daughter list holds them and their
// transformation.  Throws vgnav::Error(VGN_ERR_UNSUPPORTED) for a shape libvgnav
// has no kernel for.
inline ExportedGeometry ExportGeometry()
{
  using namespace vecgeom;
  auto &gm = GeoManager::Instance();
  ExportedGeometry e;
  const auto &lvs = gm.GetLogicalVolumesMap();
  unsigned n_lv = 0;
  for (auto const &it : lvs) n_lv = std::max(n_lv, it.first + 1);
  const unsigned n_pv = (unsigned)gm.GetPlacedVolumesCount();
  if (!gm.GetWorld() || n_lv != lvs.size())
    throw Error(VGN_ERR_ARG, "vgnav: geometry not closed, or volume ids not contiguous");
  e.lv_shape.resize(n_lv);
  e.lv_param_offset.resize(n_lv);
  std::vector<double> row;
  for (unsigned i = 0; i < n_lv; ++i) {
    LogicalVolume const *lv = lvs.at(i);
    const int type          = detail::shape_row(lv->GetUnplacedVolume(), row);
    if (type < 0) throw Error(VGN_ERR_UNSUPPORTED, std::string("vgnav: no GPU kernel for the shape of ") + lv->GetName());
    e.lv_shape[i]        = type;
    e.lv_param_offset[i] = (int32_t)e.params.size();
    e.params.insert(e.params.end(), row.begin(), row.end());
  }
  e.pv_logical.assign(n_pv, -1);
  e.pv_mother.assign(n_pv, -1);
  e.pv_transform.assign(12 * (size_t)n_pv, 0.0);
  for (unsigned i = 0; i < n_pv; ++i) {
    VPlacedVolume const *pv = gm.FindPlacedVolume((int)i);
    if (!pv) throw Error(VGN_ERR_ARG, "vgnav: placed volume ids not contiguous");
    e.pv_logical[i] = (int32_t)pv->GetLogicalVolume()->id();
    Transformation3D const *t = pv->GetTransformation();
    for (int k = 0; k < 3; ++k) e.pv_transform[12 * i + k] = t->Translation(k);
    for (int k = 0; k < 9; ++k) e.pv_transform[12 * i + 3 + k] = t->Rotation(k);
  }
  for (unsigned i = 0; i < n_lv; ++i) {
    for (VPlacedVolume const *d : lvs.at(i)->GetDaughters()) e.pv_mother[d->id()] = (int32_t)i;
    if (e.lv_shape[i] == VGN_BOOLEAN) {  // the operands belong to no mother
      const double *p = &e.params[(size_t)e.lv_param_offset[i]];
      for (int k = 1; k <= 2; ++k)
        if (p[k] >= 0 && p[k] < n_pv) e.pv_mother[(size_t)p[k]] = VGN_BOOLEAN_OPERAND;
    }
  }
  e.world_placed = (int32_t)gm.GetWorld()->id();
  return e;
}

// VecGeom navigator whose batch calls run on one GPU through libvgnav.  The scalar calls
// are VecGeom's BVH navigation on the host (hooks as in BVHNavigator.h:35-61).
class GpuBVHNavigator : public vecgeom::VNavigatorHelper<GpuBVHNavigator, false> {
  using Base = vecgeom::VNavigatorHelper<GpuBVHNavigator, false>;

public:
  using SafetyEstimator_t                          = vecgeom::BVHSafetyEstimator;
  static constexpr const char *gClassNameString = "GpuBVHNavigator";

  // Exports the closed GeoManager geometry and makes it resident on `device`.  flags:
  // VGN_PRECISION_MIXED (default) or VGN_PRECISION_FP64; results are the same.
  explicit GpuBVHNavigator(int device, int flags = VGN_PRECISION_MIXED, void *stream = nullptr)
      : Base(vecgeom::BVHSafetyEstimator::Instance()), fFlags(flags), fStream(stream)
  {
    const ExportedGeometry e = ExportGeometry();
    const vgn_geometry_desc d = e.desc();
    check(vgn_geometry_create(&d, device, &fGeom));
  }
  // Uses a geometry created by the caller (not owned).
  GpuBVHNavigator(vgn_geometry *geom, int flags, void *stream)
      : Base(vecgeom::BVHSafetyEstimator::Instance()), fGeom(geom), fOwned(false), fFlags(flags), fStream(stream)
  {
  }
  ~GpuBVHNavigator()
  {
    if (fOwned) vgn_geometry_free(fGeom);
  }
  GpuBVHNavigator(const GpuBVHNavigator &)            = delete;
  GpuBVHNavigator &operator=(const GpuBVHNavigator &) = delete;

  vgn_geometry *geometry() const { return fGeom; }

  // BVHNavigator::CheckDaughterIntersections (BVHNavigator.h:53-61), for the scalar calls
  bool CheckDaughterIntersections(vecgeom::LogicalVolume const *lvol, vecgeom::Vector3D<vecgeom::Precision> const &lp,
                                  vecgeom::Vector3D<vecgeom::Precision> const &ld,
                                  vecgeom::NavigationState const *in_state, vecgeom::NavigationState *,
                                  vecgeom::Precision &step, vecgeom::VPlacedVolume const *&hitcandidate) const
  {
    vecgeom::VPlacedVolume const *last = in_state ? in_state->GetLastExited() : nullptr;
    vecgeom::BVHManager::GetBVH(lvol)->CheckDaughterIntersections(lp, ld, step, last, hitcandidate);
    return false;
  }

  void ComputeStepsAndPropagatedStates(vecgeom::SOA3D<vecgeom::Precision> const &points,
                                       vecgeom::SOA3D<vecgeom::Precision> const &dirs,
                                       vecgeom::Precision const *step_limit,
                                       vecgeom::NavigationState const *const *in_states,
                                       vecgeom::NavigationState **out_states,
                                       vecgeom::Precision *out_steps) const override
  {
    step_gathered(points, dirs, step_limit, in_states, out_states, out_steps, nullptr, nullptr);
  }

  void ComputeStepsAndSafetiesAndPropagatedStates(vecgeom::SOA3D<vecgeom::Precision> const &points,
                                                  vecgeom::SOA3D<vecgeom::Precision> const &dirs,
                                                  vecgeom::Precision const *step_limit,
                                                  vecgeom::NavStatePool const &in_states,
                                                  vecgeom::NavStatePool &out_states, vecgeom::Precision *out_steps,
                                                  bool const *calcsafeties,
                                                  vecgeom::Precision *out_safeties) const override
  {
    // a NavStatePool of NavStateIndex is one contiguous array of 12-byte states
    // (NavStatePool.h:153-161, NavStateIndex.h:95-99)
    const int64_t n = (int64_t)points.size();
    if (n == 0) return;
    const auto *in = reinterpret_cast<const vgn_state *>(in_states[0]);
    auto *out      = reinterpret_cast<vgn_state *>(out_states[0]);
    step(n, points, dirs, step_limit, in, out, out_steps, calcsafeties, out_safeties);
  }

  void ComputeStepsAndSafetiesAndPropagatedStates(vecgeom::SOA3D<vecgeom::Precision> const &points,
                                                  vecgeom::SOA3D<vecgeom::Precision> const &dirs,
                                                  vecgeom::Precision const *step_limit,
                                                  vecgeom::NavigationState const *const *in_states,
                                                  vecgeom::NavigationState **out_states,
                                                  vecgeom::Precision *out_steps, bool const *calcsafeties,
                                                  vecgeom::Precision *out_safeties) const override
  {
    step_gathered(points, dirs, step_limit, in_states, out_states, out_steps, calcsafeties, out_safeties);
  }

private:
  // per-track calcsafeties: safeties are computed for the batch when any track asks and
  // written as 0 for the others, as the reference's masked safety does (VNavigator.h:419-426)
  void step(int64_t n, vecgeom::SOA3D<vecgeom::Precision> const &points,
            vecgeom::SOA3D<vecgeom::Precision> const &dirs, vecgeom::Precision const *step_limit, const vgn_state *in,
            vgn_state *out, vecgeom::Precision *out_steps, bool const *calcsafeties,
            vecgeom::Precision *out_safeties) const
  {
    bool any = false;
    for (int64_t i = 0; calcsafeties && out_safeties && i < n && !any; ++i) any = calcsafeties[i];
    check(vgn_compute_step_batch(fGeom, n, points.x(), points.y(), points.z(), dirs.x(), dirs.y(), dirs.z(),
                                 step_limit, in, out, out_steps, any ? out_safeties : nullptr, fFlags, fStream));
    if (out_safeties && calcsafeties)
      for (int64_t i = 0; i < n; ++i)
        if (!calcsafeties[i]) out_safeties[i] = 0.;
  }

  void step_gathered(vecgeom::SOA3D<vecgeom::Precision> const &points, vecgeom::SOA3D<vecgeom::Precision> const &dirs,
                     vecgeom::Precision const *step_limit, vecgeom::NavigationState const *const *in_states,
                     vecgeom::NavigationState **out_states, vecgeom::Precision *out_steps, bool const *calcsafeties,
                     vecgeom::Precision *out_safeties) const
  {
    const int64_t n = (int64_t)points.size();
    if (n == 0) return;
    std::vector<vgn_state> in((size_t)n), out((size_t)n);
    for (int64_t i = 0; i < n; ++i) std::memcpy(&in[(size_t)i], in_states[i], sizeof(vgn_state));
    step(n, points, dirs, step_limit, in.data(), out.data(), out_steps, calcsafeties, out_safeties);
    for (int64_t i = 0; i < n; ++i) std::memcpy(out_states[i], &out[(size_t)i], sizeof(vgn_state));
  }

  vgn_geometry *fGeom = nullptr;
  bool fOwned         = true;
  int fFlags;
  void *fStream;
};

} // namespace vgnav

#endif
