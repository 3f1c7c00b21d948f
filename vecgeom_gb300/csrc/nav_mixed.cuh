// nav_mixed.cuh -- exact-decision mixed-precision BVH traversal.
//
// GB300 executes FP64 at a small fraction of its FP32 rate.  The reference's
// traversal spends most of its FP64 work on box tests whose only outcome is a
// yes/no decision (visit a node, test a candidate, which child first).  Here
// every such decision is first taken in FP32 interval arithmetic with directed
// rounding (__fsub_rd, __fmul_ru, ...): the interval provably contains the
// value the FP64 code would compute, so when it lies entirely on one side of
// the threshold the FP64 decision is known.  Only when the interval straddles
// the threshold is the quantity recomputed in FP64.  Distances that reach the
// output (DistanceToIn/Out, SafetyToIn/Out, transforms) are always FP64.  The
// result is therefore bit-identical to the all-FP64 traversal: same visit
// order, same candidates, same tie-breaking.
#pragma once

#include "nav_device.cuh"

namespace vgn {
namespace dev {

struct FI {
  float lo, hi;
};

// tri-state decisions
enum : int { kNo = 0, kYes = 1, kMaybe = 2 };

__device__ __forceinline__ FI fi(double x) { return FI{__double2float_rd(x), __double2float_ru(x)}; }
__device__ __forceinline__ int fi_lt(FI a, FI b) { return a.hi < b.lo ? kYes : (a.lo >= b.hi ? kNo : kMaybe); }
__device__ __forceinline__ int fi_le(FI a, FI b) { return a.hi <= b.lo ? kYes : (a.lo > b.hi ? kNo : kMaybe); }
__device__ __forceinline__ int fi_ge0(FI a) { return a.lo >= 0.f ? kYes : (a.hi < 0.f ? kNo : kMaybe); }
__device__ __forceinline__ int and3(int a, int b, int c)
{
  if (a == kNo || b == kNo || c == kNo) return kNo;
  return (a == kYes && b == kYes && c == kYes) ? kYes : kMaybe;
}

__device__ __forceinline__ FI fi_sub(FI a, FI b) { return FI{__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)}; }
__device__ __forceinline__ FI fi_add(FI a, FI b) { return FI{__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ FI fi_mul(FI a, FI b)
{
  const float l = fminf(fminf(__fmul_rd(a.lo, b.lo), __fmul_rd(a.lo, b.hi)),
                        fminf(__fmul_rd(a.hi, b.lo), __fmul_rd(a.hi, b.hi)));
  const float h = fmaxf(fmaxf(__fmul_ru(a.lo, b.lo), __fmul_ru(a.lo, b.hi)),
                        fmaxf(__fmul_ru(a.hi, b.lo), __fmul_ru(a.hi, b.hi)));
  return FI{l, h};
}
// product with an interval b of known sign (b does not contain 0)
__device__ __forceinline__ FI fi_mul_signed(FI a, FI b, bool bneg)
{
  if (!bneg) return FI{__fmul_rd(a.lo, a.lo >= 0.f ? b.lo : b.hi), __fmul_ru(a.hi, a.hi >= 0.f ? b.hi : b.lo)};
  return FI{__fmul_rd(a.hi, a.hi >= 0.f ? b.lo : b.hi), __fmul_ru(a.lo, a.lo >= 0.f ? b.hi : b.lo)};
}
__device__ __forceinline__ FI fi_abs(FI a)
{
  if (a.lo >= 0.f) return a;
  if (a.hi <= 0.f) return FI{-a.hi, -a.lo};
  return FI{0.f, fmaxf(-a.lo, a.hi)};
}
__device__ __forceinline__ FI fi_max(FI a, FI b) { return FI{fmaxf(a.lo, b.lo), fmaxf(a.hi, b.hi)}; }
__device__ __forceinline__ FI fi_min(FI a, FI b) { return FI{fminf(a.lo, b.lo), fminf(a.hi, b.hi)}; }

// Per-track ray in FP32 intervals plus the FP64 inverse direction, made on first need.
struct MixedRay {
  FI p[3];
  FI inv[3];
  bool neg[3];
  D3 lp, ld;
  D3 inv64;
  bool have_inv64;
};

__device__ __forceinline__ void make_ray(MixedRay &r, D3 lp, D3 ld)
{
  r.lp = lp;
  r.ld = ld;
  r.p[0] = fi(lp.x);
  r.p[1] = fi(lp.y);
  r.p[2] = fi(lp.z);
  const double d[3] = {nonzero(ld.x), nonzero(ld.y), nonzero(ld.z)};  // Global.h:174-178
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const FI di = fi(d[k]);  // same sign at both ends: |d| >= 1e-30
    r.inv[k]    = FI{__frcp_rd(di.hi), __frcp_ru(di.lo)};  // 1/x decreases on each half line
    r.neg[k]    = di.hi < 0.f;
  }
  r.have_inv64 = false;
}

__device__ __forceinline__ D3 ray_inv64(MixedRay &r)
{
  if (!r.have_inv64) {
    r.inv64      = d3(1.0 / nonzero(r.ld.x), 1.0 / nonzero(r.ld.y), 1.0 / nonzero(r.ld.z));
    r.have_inv64 = true;
  }
  return r.inv64;
}

// Interval of AABB::ComputeIntersectionInvDir's (tmin, tmax).  The FP64 code's
// swap leaves t(min side) <= t(max side) per axis; which side is "near" only
// depends on the sign of the inverse direction, by monotonicity of rounding.
__device__ __forceinline__ void islab(const float *mn_lo, const float *mn_hi, const float *mx_lo, const float *mx_hi,
                                      const MixedRay &r, FI &tmin, FI &tmax)
{
  FI near[3], far[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const FI a0 = FI{__fsub_rd(__ldg(mn_lo + k), r.p[k].hi), __fsub_ru(__ldg(mn_hi + k), r.p[k].lo)};
    const FI a1 = FI{__fsub_rd(__ldg(mx_lo + k), r.p[k].hi), __fsub_ru(__ldg(mx_hi + k), r.p[k].lo)};
    const FI t0 = fi_mul_signed(a0, r.inv[k], r.neg[k]);
    const FI t1 = fi_mul_signed(a1, r.inv[k], r.neg[k]);
    near[k]     = r.neg[k] ? t1 : t0;
    far[k]      = r.neg[k] ? t0 : t1;
  }
  tmin = fi_max(fi_max(near[0], near[1]), near[2]);
  const FI f = fi_min(fi_min(far[0], far[1]), far[2]);
  // times (1 + 2 eps): the exact factor lies in [1, 1 + 2^-23]
  constexpr float kUp = 1.00000011920928955078125f;
  tmax = FI{f.lo >= 0.f ? f.lo : __fmul_rd(f.lo, kUp), f.hi >= 0.f ? __fmul_ru(f.hi, kUp) : f.hi};
}

// tmin <= tmax && tmax >= 0 && tmin < step  (BVH.h:113, 130-131)
__device__ __forceinline__ int slab_decision(FI tmin, FI tmax, FI step)
{
  return and3(fi_le(tmin, tmax), fi_ge0(tmax), fi_lt(tmin, step));
}

// Interval of AABB::Safety (AABB.h:81): max_k(|p_k - c_k| - hs_k)
__device__ __forceinline__ FI isafety(const ISafe &s, const MixedRay &r)
{
  FI m;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const FI c  = FI{__ldg(&s.c_lo[k]), __ldg(&s.c_hi[k])};
    const FI hs = FI{__ldg(&s.hs_lo[k]), __ldg(&s.hs_hi[k])};
    const FI v  = fi_sub(fi_abs(fi_sub(r.p[k], c)), hs);
    m           = k == 0 ? v : fi_max(m, v);
  }
  return m;
}

// Interval of a box daughter's SafetyToIn: placement transform then
// BoxImplementation::SafetyToIn (BoxImplementation.h:153-158).
__device__ __forceinline__ FI ibox_safety_in(const IXForm &x, const MixedRay &r)
{
  FI t[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) t[k] = fi_sub(r.p[k], FI{__ldg(&x.t_lo[k]), __ldg(&x.t_hi[k])});
  FI m;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    FI l = fi_mul(t[0], FI{__ldg(&x.r_lo[i]), __ldg(&x.r_hi[i])});
    l    = fi_add(l, fi_mul(t[1], FI{__ldg(&x.r_lo[3 + i]), __ldg(&x.r_hi[3 + i])}));
    l    = fi_add(l, fi_mul(t[2], FI{__ldg(&x.r_lo[6 + i]), __ldg(&x.r_hi[6 + i])}));
    const FI v = fi_sub(fi_abs(l), FI{__ldg(&x.h_lo[i]), __ldg(&x.h_hi[i])});
    m          = i == 0 ? v : fi_max(m, v);
  }
  return m;
}

// BVH::CheckDaughterIntersections (BVH.h:96-146) with interval decisions
__device__ __forceinline__ bool bvh_check_daughters_mixed(const GeomView &g, const LVRec &lv, MixedRay &r,
                                                          double &step, int last, int &hit)
{
  unsigned stack[kStackSize];
  int sp   = 1;
  stack[0] = 0;
  FI stepI = fi(step);
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  const PrimRec *prims    = g.prims + lv.prims_off;
  do {
    const unsigned id = stack[--sp];
    const int nchild  = __ldg(&inodes[id].nchild);
    if (nchild >= 0) {
      const int off = __ldg(&inodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const IPrimSlab &q = iprims[off + i];
        FI tmin, tmax;
        islab(q.mn_lo, q.mn_hi, q.mx_lo, q.mx_hi, r, tmin, tmax);
        int dec = slab_decision(tmin, tmax, stepI);
        if (dec == kMaybe) {
          double a, b;
          slab(prims[off + i].mn, prims[off + i].mx, r.lp, ray_inv64(r), a, b);
          dec = (a <= b && b >= 0.0 && a < step) ? kYes : kNo;
        }
        if (dec == kYes) {
          const int vol     = __ldg(&q.pv);
          const double dist = pv_dist_in(g, vol, r.lp, r.ld);
          if (dist < step && !(dist <= 0.0 && vol == last)) {
            step  = dist;
            hit   = vol;
            stepI = fi(step);
          }
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      FI tminL, tmaxL, tminR, tmaxR;
      islab(inodes[L].mn_lo, inodes[L].mn_hi, inodes[L].mx_lo, inodes[L].mx_hi, r, tminL, tmaxL);
      islab(inodes[R].mn_lo, inodes[R].mn_hi, inodes[R].mx_lo, inodes[R].mx_hi, r, tminR, tmaxR);
      int trL = slab_decision(tminL, tmaxL, stepI);
      int trR = slab_decision(tminR, tmaxR, stepI);
      int rfirst = fi_lt(tminR, tminL);
      if (trL == kMaybe || trR == kMaybe || rfirst == kMaybe) {
        const D3 inv = ray_inv64(r);
        double a, b, c, d;
        slab(nodes[L].mn, nodes[L].mx, r.lp, inv, a, b);
        slab(nodes[R].mn, nodes[R].mx, r.lp, inv, c, d);
        trL    = (a <= b && b >= 0.0 && a < step) ? kYes : kNo;
        trR    = (c <= d && d >= 0.0 && c < step) ? kYes : kNo;
        rfirst = c < a ? kYes : kNo;
      }
      if (sp + 2 > kStackSize) {
        raise_error(g, kErrStack);
        return false;
      }
      if (rfirst == kYes) {
        if (trR == kYes) stack[sp++] = R;
        if (trL == kYes) stack[sp++] = L;
      } else {
        if (trL == kYes) stack[sp++] = L;
        if (trR == kYes) stack[sp++] = R;
      }
    }
  } while (sp > 0);
  return true;
}

// BVH::ComputeSafety (BVH.h:172-209) with interval decisions; a box daughter
// whose SafetyToIn interval cannot go below the current safety is skipped
// without any FP64 work (it would not change the result either way).
__device__ __forceinline__ double bvh_safety_mixed(const GeomView &g, const LVRec &lv, const MixedRay &r,
                                                   double safety)
{
  unsigned stack[kStackSize];
  int sp   = 1;
  stack[0] = 0;
  FI safI  = fi(safety);
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const ISafe *isafe_n    = g.inode_safe + lv.nodes_off;
  const ISafe *isafe_p    = g.iprim_safe + lv.prims_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  const PrimRec *prims    = g.prims + lv.prims_off;
  do {
    const unsigned id = stack[--sp];
    const int nchild  = __ldg(&inodes[id].nchild);
    if (nchild >= 0) {
      const int off = __ldg(&inodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const int vol = __ldg(&iprims[off + i].pv);
        const IXForm &x = g.ixf[vol];
        if (__ldg(&x.shape) == kBox && fi_lt(ibox_safety_in(x, r), safI) == kNo) continue;
        int dec = fi_lt(isafety(isafe_p[off + i], r), safI);
        if (dec == kMaybe) dec = box_safety(prims[off + i].mn, prims[off + i].mx, r.lp) < safety ? kYes : kNo;
        if (dec == kYes) {
          const double dist = pv_safe_in(g, vol, r.lp);
          if (dist < safety) {
            safety = dist;
            safI   = fi(safety);
          }
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      const FI sL = isafety(isafe_n[L], r);
      const FI sR = isafety(isafe_n[R], r);
      int trL = fi_lt(sL, safI), trR = fi_lt(sR, safI), rfirst = fi_lt(sR, sL);
      if (trL == kMaybe || trR == kMaybe || rfirst == kMaybe) {
        const double a = box_safety(nodes[L].mn, nodes[L].mx, r.lp);
        const double b = box_safety(nodes[R].mn, nodes[R].mx, r.lp);
        trL    = a < safety ? kYes : kNo;
        trR    = b < safety ? kYes : kNo;
        rfirst = b < a ? kYes : kNo;
      }
      if (sp + 2 > kStackSize) {
        raise_error(g, kErrStack);
        return safety;
      }
      if (rfirst == kYes) {
        if (trR == kYes) stack[sp++] = R;
        if (trL == kYes) stack[sp++] = L;
      } else {
        if (trL == kYes) stack[sp++] = L;
        if (trR == kYes) stack[sp++] = R;
      }
    }
  } while (sp > 0);
  return safety;
}

// p >= mn && p <= mx per axis (AABB::Contains, AABB.h:69-72) as a tri-state
__device__ __forceinline__ int icontains(const float *mn_lo, const float *mn_hi, const float *mx_lo,
                                         const float *mx_hi, const FI *p)
{
  int res = kYes;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float a = __ldg(mn_lo + k), b = __ldg(mn_hi + k), c = __ldg(mx_lo + k), d = __ldg(mx_hi + k);
    const int ge = p[k].lo >= b ? kYes : (p[k].hi < a ? kNo : kMaybe);
    const int le = p[k].hi <= c ? kYes : (p[k].lo > d ? kNo : kMaybe);
    if (ge == kNo || le == kNo) return kNo;
    if (ge == kMaybe || le == kMaybe) res = kMaybe;
  }
  return res;
}

// BVH::LevelLocate(exclvol, localpoint, pvol, daughterlocalpoint) (BVH.h:255-285)
__device__ __forceinline__ bool bvh_level_locate_mixed(const GeomView &g, const LVRec &lv, int excl, D3 lp,
                                                       int &pvol, D3 &dlp)
{
  unsigned stack[kStackSize];
  int sp   = 1;
  stack[0] = 0;
  const FI p[3] = {fi(lp.x), fi(lp.y), fi(lp.z)};
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  const PrimRec *prims    = g.prims + lv.prims_off;
  do {
    const unsigned id = stack[--sp];
    const int nchild  = __ldg(&inodes[id].nchild);
    if (nchild >= 0) {
      const int off = __ldg(&inodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const IPrimSlab &q = iprims[off + i];
        int dec = icontains(q.mn_lo, q.mn_hi, q.mx_lo, q.mx_hi, p);
        if (dec == kMaybe) dec = box_contains_pt(prims[off + i].mn, prims[off + i].mx, lp) ? kYes : kNo;
        if (dec == kYes) {
          const int vol = __ldg(&q.pv);
          if (vol != excl && pv_contains(g, vol, lp, dlp)) {
            pvol = vol;
            return true;
          }
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      if (sp + 2 > kStackSize) {
        raise_error(g, kErrStack);
        return false;
      }
      int cL = icontains(inodes[L].mn_lo, inodes[L].mn_hi, inodes[L].mx_lo, inodes[L].mx_hi, p);
      if (cL == kMaybe) cL = box_contains_pt(nodes[L].mn, nodes[L].mx, lp) ? kYes : kNo;
      if (cL == kYes) stack[sp++] = L;
      int cR = icontains(inodes[R].mn_lo, inodes[R].mn_hi, inodes[R].mx_lo, inodes[R].mx_hi, p);
      if (cR == kMaybe) cR = box_contains_pt(nodes[R].mn, nodes[R].mx, lp) ? kYes : kNo;
      if (cR == kYes) stack[sp++] = R;
    }
  } while (sp > 0);
  return false;
}

}  // namespace dev
}  // namespace vgn
