// nav_step.cuh -- one navigation step per thread, for both kernel sets.
//
// MIXED = false: every box test in FP64 (the "plain" form).
// MIXED = true : box tests decided in FP32 intervals (nav_mixed.cuh).
// Both produce bit-identical steps, safeties and states.
#pragma once

#include "nav_mixed.cuh"

namespace vgn {
namespace dev {
inline namespace VGN_KSET {

template <bool MIXED>
__device__ __forceinline__ bool level_locate(const GeomView &g, const LVRec &lv, int excl, D3 lp, int &pvol, D3 &dlp)
{
  return MIXED ? bvh_level_locate_mixed(g, lv, excl, lp, pvol, dlp) : bvh_level_locate(g, lv, excl, lp, pvol, dlp);
}

// GlobalLocator::LocateGlobalPoint (GlobalLocator.h:35-82), BVHLevelLocator attached
template <bool MIXED>
__device__ __forceinline__ int locate_global_point(const GeomView &g, int vol, D3 point, uint32_t &path, bool top)
{
  int cand = vol;
  D3 cur   = point;
  if (top) cand = pv_unplaced_contains(g, vol, point) ? vol : -1;
  if (cand >= 0) {
    path     = ni_push(g, path, cand);
    LVRec lv = load_lv(g, pv_lv(g, cand));
    bool godeeper = true;
    int guard     = 0;
    while (lv.nd > 0 && godeeper) {
      if (++guard > g.level_limit) {
        raise_error(g, kErrRelocate);
        break;
      }
      int pv;
      D3 tp;
      godeeper = level_locate<MIXED>(g, lv, -1, cur, pv, tp);
      if (godeeper) {
        path = ni_push(g, path, pv);
        cand = pv;
        lv   = load_lv(g, pv_lv(g, cand));
        cur  = tp;
      }
    }
  }
  return cand >= 0 ? ni_top(g, path) : -1;
}

// GlobalLocator::LocateGlobalPointExclVolume (GlobalLocator.h:88-135)
template <bool MIXED>
__device__ __forceinline__ void locate_global_point_excl(const GeomView &g, int vol, int excl, D3 point,
                                                         uint32_t &path)
{
  int cand = vol;
  D3 cur   = point;
  path     = ni_push(g, path, cand);
  LVRec lv = load_lv(g, pv_lv(g, cand));
  bool godeeper = true;
  int guard     = 0;
  while (lv.nd > 0 && godeeper) {
    if (++guard > g.level_limit) {
      raise_error(g, kErrRelocate);
      break;
    }
    D3 tp;
    godeeper = level_locate<MIXED>(g, lv, excl, cur, cand, tp);
    if (godeeper) {
      lv   = load_lv(g, pv_lv(g, cand));
      cur  = tp;
      path = ni_push(g, path, cand);
    }
  }
}

// GlobalLocator::RelocatePointFromPathForceDifferent (GlobalLocator.h:171-200)
template <bool MIXED>
__device__ __forceinline__ void relocate_force_different(const GeomView &g, D3 lp, uint32_t &path)
{
  int cm          = ni_top(g, path);
  const int entry = cm;
  if (cm < 0) return;
  D3 tmp    = lp;
  int guard = 0;
  while (cm >= 0) {
    if (++guard > g.level_limit + 1) {
      raise_error(g, kErrRelocate);
      return;
    }
    if (cm == entry || !pv_unplaced_contains(g, cm, tmp)) {
      path = ni_pop(g, path);
      PvXf x;
      load_pv_xf(g, cm, x);
      tmp = xf_inverse(x.t, x.r, tmp);
      cm  = ni_top(g, path);
    } else
      break;
  }
  if (cm >= 0) {
    path = ni_pop(g, path);
    locate_global_point_excl<MIXED>(g, cm, entry, tmp, path);
  }
}

// VNavigatorHelper::Relocate (VNavigator.h:1070-1091)
template <bool MIXED>
__device__ __forceinline__ void relocate(const GeomView &g, D3 pab, const State &in, State &out)
{
  if (ni_top(g, out.nav_ind) == ni_top(g, in.nav_ind)) {
    relocate_force_different<MIXED>(g, pab, out.nav_ind);
  } else {
    const int nextvol = ni_top(g, out.nav_ind);
    out.nav_ind       = ni_pop(g, out.nav_ind);
    PvXf x;
    load_pv_xf(g, nextvol, x);
    locate_global_point<MIXED>(g, nextvol, xf_point(x.t, x.r, pab), out.nav_ind, false);
  }
}

// BVHSafetyEstimator::ComputeSafetyForLocalPoint (BVHSafetyEstimator.h:38-46)
template <bool MIXED>
__device__ __forceinline__ double safety_local(const GeomView &g, const LVRec &lv, D3 lp, D3 ld)
{
  double safety = shape_safe_out(lv.shape, g.shape + lv.shape_row, lp);
  if (safety > 0.0 && lv.nd > 0) {
    if (MIXED) {
      MixedRay r;
      make_ray(r, lp, ld);
      safety = bvh_safety_mixed(g, lv, r, safety);
    } else {
      safety = bvh_safety(g, lv, lp, safety);
    }
  }
  return safety;
}

// Start of a step: the input state's global matrix, the local point and direction, the
// volume and the mother's DistanceToOut, given the step limit (VNavigator.h:241-249, 444-458;
// BVHNavigator.h:53-61; a boolean mother hands it to its operands).
__device__ __forceinline__ void step_begin(const GeomView &g, D3 gp, D3 gd, double slimit, const State &in, D3 &lp,
                                           D3 &ld, LVRec &lv, double &step)
{
  Xf m;
  top_matrix(g, in.nav_ind, m);
  lp            = xf_point(m.t, m.r, gp);
  ld            = xf_dir(m.r, gd);
  const int pv  = ni_top(g, in.nav_ind);
  lv            = load_lv(g, pv_lv(g, pv));
  step          = shape_dist_out(lv.shape, g.shape + lv.shape_row, lp, ld, slimit);
  if (step < 0.) step = 0.;
}

// End of a step, given the daughters' verdict (step, hit): PrepareOutState
// (VNavigator.h:192-235) and MovePointAfterBoundary (168-173) with relocation.
template <bool MIXED>
__device__ __forceinline__ double step_finish(const GeomView &g, D3 lp, D3 ld, double slimit, const State &in,
                                              State &out, bool reloc, double step, int hit)
{
  out = in;
  if (step == kInfLength && slimit > 0.) {
    out.on_boundary = 1;
    out.nav_ind     = ni_pop(g, out.nav_ind);
    return kTolerance;
  }
  if (step > slimit) {
    out.on_boundary = 0;
    return slimit;
  }
  out.on_boundary = 1;
  out.last_exited = out.nav_ind;
  if (hit >= 0) out.nav_ind = ni_push(g, out.nav_ind, hit);
  if (step < 0.) step = 0.;
  if (!reloc) return step;
  const double s = step + 1E-6;
  relocate<MIXED>(g, d3(lp.x + s * ld.x, lp.y + s * ld.y, lp.z + s * ld.z), in, out);
  return step;
}

// ComputeStepAndPropagatedState (VNavigator.h:436-492) with PrepareOutState
// (VNavigator.h:192-235) and MovePointAfterBoundary (168-173).  The safety of
// ComputeStepAndSafetyAndPropagatedState (VNavigator.h:1014-1064) is taken at the
// input state and does not affect the step: the safety pass (safety_local) computes it.
template <bool MIXED>
__device__ __forceinline__ double nav_step(const GeomView &g, D3 gp, D3 gd, double slimit, const State &in,
                                           State &out, bool reloc)
{
  D3 lp, ld;
  LVRec lv;
  double step;
  step_begin(g, gp, gd, slimit, in, lp, ld, lv, step);
  int hit = -1;
  if (MIXED) {
    MixedRay r;
    make_ray(r, lp, ld);
    if (lv.nd > 0) bvh_check_daughters_mixed(g, lv, r, step, ni_top(g, in.last_exited), hit);
  } else {
    if (lv.nd > 0) bvh_check_daughters(g, lv, lp, ld, step, ni_top(g, in.last_exited), hit);
  }
  return step_finish<MIXED>(g, lp, ld, slimit, in, out, reloc, step, hit);
}

}  // namespace VGN_KSET
}  // namespace dev
}  // namespace vgn
