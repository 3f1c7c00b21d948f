// nav_device.cuh -- device-side navigation: navigation-index decoding,
// transforms, BVH traversal (FP64), relocation, safety and point location.
//
// One thread owns one track for the whole step: global->local transform,
// mother DistanceToOut, BVH traversal with leaf DistanceToIn through a
// switch on the shape type (no virtual calls), PrepareOutState, and the
// relocation after the boundary.  Every loop is bounded; overflow of the
// traversal stack or of the geometry depth sets a bit in the status word and
// ends the track's work instead of trapping.
#pragma once

#include "shapes_fp64.cuh"

namespace vgn {
namespace dev {
inline namespace VGN_KSET {

struct State {
  uint32_t nav_ind, last_exited;
  uint32_t on_boundary;
};

__device__ __forceinline__ void raise_error(const GeomView &g, uint32_t bit) { atomicOr(g.status, bit); }

// ---- NavStateIndex decoding (NavStateIndex.h:136-265) ----
__device__ __forceinline__ uint32_t ni_word(const GeomView &g, uint32_t i) { return __ldg(g.navind + i); }
__device__ __forceinline__ int ni_top(const GeomView &g, uint32_t ni) { return ni > 0 ? (int)ni_word(g, ni + 1) : -1; }
__device__ __forceinline__ uint32_t ni_pop(const GeomView &g, uint32_t ni) { return ni > 0 ? ni_word(g, ni) : 0u; }
__device__ __forceinline__ uint32_t ni_push(const GeomView &g, uint32_t ni, int pv)
{
  return ni > 0 ? ni_word(g, ni + 3 + (uint32_t)__ldg(&g.pv[pv].child_id)) : 1u;
}
// a navigation index supplied by the caller must start a state record of the table
__device__ __forceinline__ bool ni_valid(const GeomView &g, uint32_t ni)
{
  return ni > 0 && ni < g.navind_words && ((__ldg(g.node_start + (ni >> 5)) >> (ni & 31)) & 1u);
}

struct Xf {
  double t[3];
  double r[9];
};

// Transformation3D::MultiplyFromRight (Transformation3D.h:878-946) on a transform with its
// identity / translation / rotation flags (flags: kXfTrans | kXfRot, none = identity)
__device__ __forceinline__ void xf_mul_right(Xf &m, int &mflags, const double *rt, const double *rr, int rflags)
{
  if (rflags == 0) return;
  if (rflags & kXfTrans) {
    mflags |= kXfTrans;
#pragma unroll
    for (int row = 0; row < 3; ++row) {
      m.t[row] += m.r[3 * row + 0] * rt[0];
      m.t[row] += m.r[3 * row + 1] * rt[1];
      m.t[row] += m.r[3 * row + 2] * rt[2];
    }
  }
  if (rflags & kXfRot) {
    mflags |= kXfRot;
#pragma unroll
    for (int row = 0; row < 3; ++row) {
      double *r      = m.r + 3 * row;
      const double x = r[0], y = r[1], z = r[2];
      r[0] = x * rr[0];
      r[1] = x * rr[1];
      r[2] = x * rr[2];
      r[0] += y * rr[3];
      r[1] += y * rr[4];
      r[2] += y * rr[5];
      r[0] += z * rr[6];
      r[1] += z * rr[7];
      r[2] += z * rr[8];
    }
  }
}

__device__ __forceinline__ void xf_set_identity(Xf &m)
{
  m.t[0] = m.t[1] = m.t[2] = 0.;
  m.r[0] = 1.; m.r[1] = 0.; m.r[2] = 0.;
  m.r[3] = 0.; m.r[4] = 1.; m.r[5] = 0.;
  m.r[6] = 0.; m.r[7] = 0.; m.r[8] = 1.;
}

// TopMatrixImpl (NavStateIndex.h:232-265): the global-to-local matrix of a state.  Levels
// without a cached matrix (deeper than the table's cache depth) contribute their placement
// transforms, t.MultiplyFromRight(trans), walking up to the first cached ancestor, whose
// matrix is applied last; with every level cached the first node's matrix is the result.
__device__ __forceinline__ void top_matrix(const GeomView &g, uint32_t ni, Xf &m)
{
  xf_set_identity(m);
  int mflags = 0;
  if (ni == 0) return;
  uint32_t w    = ni_word(g, ni + 2);
  uint32_t hasm = (w >> 8) & 0xffu;
  while (!(hasm & 0x04u)) {  // no cached matrix at this level
    const int pv = ni_top(g, ni);
    Xf t;
    const double *x = &g.pv[pv].xf.t[0];
#pragma unroll
    for (int i = 0; i < 3; ++i) t.t[i] = __ldg(x + i);
#pragma unroll
    for (int i = 0; i < 9; ++i) t.r[i] = __ldg(x + 3 + i);
    int tflags = __ldg(&g.pv[pv].xf_flags);
    xf_mul_right(t, tflags, m.t, m.r, mflags);
    m      = t;
    mflags = tflags;
    ni     = ni_pop(g, ni);
    if (ni == 0) return;
    w    = ni_word(g, ni + 2);
    hasm = (w >> 8) & 0xffu;
  }
  if ((hasm & 0x03u) == 0) return;
  const uint32_t nd = w >> 16;
  uint32_t idx      = ni + 3 + nd + ((nd + 1) & 1);
  if ((idx * 4) % 8 != 0) idx += 1;
  const double *a = reinterpret_cast<const double *>(g.navind + idx);
  Xf t;
  xf_set_identity(t);
  int tflags = ((hasm & 0x02u) ? kXfTrans : 0) | ((hasm & 0x01u) ? kXfRot : 0);  // Transformation3D::Set
  if (hasm & 0x02u) {
    t.t[0] = __ldg(a + 0);
    t.t[1] = __ldg(a + 1);
    t.t[2] = __ldg(a + 2);
  }
  if (hasm & 0x01u) {
#pragma unroll
    for (int i = 0; i < 9; ++i) t.r[i] = __ldg(a + 3 + i);
  }
  xf_mul_right(t, tflags, m.t, m.r, mflags);
  m = t;
}

// Transform<kGeneric,kGeneric>: xf_point and xf_dir (shapes_fp64.cuh)

// InverseTransform (Transformation3D.h:793-827)
__device__ __forceinline__ D3 xf_inverse(const double *t, const double *r, D3 l)
{
  double a = t[0], b = t[1], c = t[2];
  a += l.x * r[0];
  a += l.y * r[1];
  a += l.z * r[2];
  b += l.x * r[3];
  b += l.y * r[4];
  b += l.z * r[5];
  c += l.x * r[6];
  c += l.y * r[7];
  c += l.z * r[8];
  return d3(a, b, c);
}

// placement transform of placed volume pv, read through the read-only cache
struct PvXf {
  double t[3];
  double r[9];
};
__device__ __forceinline__ void load_pv_xf(const GeomView &g, int pv, PvXf &x)
{
  const double *src = &g.pv[pv].xf.t[0];
#pragma unroll
  for (int i = 0; i < 3; ++i) x.t[i] = __ldg(src + i);
#pragma unroll
  for (int i = 0; i < 9; ++i) x.r[i] = __ldg(src + 3 + i);
}

__device__ __forceinline__ const double *pv_row(const GeomView &g, int pv, int &type)
{
  type = __ldg(&g.pv[pv].shape);
  return g.shape + __ldg(&g.pv[pv].shape_row);
}

// placed DistanceToIn / SafetyToIn / Contains (SpecializedPlacedVolImplHelper.h:118-175)
__device__ __forceinline__ double pv_dist_in(const GeomView &g, int pv, D3 p, D3 d, double stepmax)
{
  PvXf x;
  load_pv_xf(g, pv, x);
  int type;
  const double *row = pv_row(g, pv, type);
  return shape_dist_in(type, row, xf_point(x.t, x.r, p), xf_dir(x.r, d), stepmax);
}

__device__ __forceinline__ double pv_safe_in(const GeomView &g, int pv, D3 p)
{
  PvXf x;
  load_pv_xf(g, pv, x);
  int type;
  const double *row = pv_row(g, pv, type);
  return shape_safe_in(type, row, xf_point(x.t, x.r, p));
}

__device__ __forceinline__ bool pv_contains(const GeomView &g, int pv, D3 p, D3 &lp)
{
  PvXf x;
  load_pv_xf(g, pv, x);
  int type;
  const double *row = pv_row(g, pv, type);
  lp                = xf_point(x.t, x.r, p);
  return shape_contains(type, row, lp);
}

__device__ __forceinline__ bool pv_unplaced_contains(const GeomView &g, int pv, D3 p)
{
  int type;
  const double *row = pv_row(g, pv, type);
  return shape_contains(type, row, p);
}

// AABB::ComputeIntersectionInvDir (AABB.h:136-154)
__device__ __forceinline__ void slab(const double *mn, const double *mx, D3 p, D3 inv, double &tmin, double &tmax)
{
  double a0 = (__ldg(mn + 0) - p.x) * inv.x, b0 = (__ldg(mx + 0) - p.x) * inv.x;
  double a1 = (__ldg(mn + 1) - p.y) * inv.y, b1 = (__ldg(mx + 1) - p.y) * inv.y;
  double a2 = (__ldg(mn + 2) - p.z) * inv.z, b2 = (__ldg(mx + 2) - p.z) * inv.z;
  double s;
  if (a0 > b0) { s = a0; a0 = b0; b0 = s; }
  if (a1 > b1) { s = a1; a1 = b1; b1 = s; }
  if (a2 > b2) { s = a2; a2 = b2; b2 = s; }
  tmin = max3(a0, a1, a2);
  tmax = min3(b0, b1, b2) * (1. + 2 * kEpsilon);
}

// AABB::Safety (AABB.h:81)
__device__ __forceinline__ double box_safety(const double *mn, const double *mx, D3 p)
{
  const double mn0 = __ldg(mn + 0), mn1 = __ldg(mn + 1), mn2 = __ldg(mn + 2);
  const double mx0 = __ldg(mx + 0), mx1 = __ldg(mx + 1), mx2 = __ldg(mx + 2);
  const double c0 = 0.5 * (mx0 + mn0), c1 = 0.5 * (mx1 + mn1), c2 = 0.5 * (mx2 + mn2);
  const double s0 = mx0 - mn0, s1 = mx1 - mn1, s2 = mx2 - mn2;
  return max3(fabs(p.x - c0) - 0.5 * s0, fabs(p.y - c1) - 0.5 * s1, fabs(p.z - c2) - 0.5 * s2);
}

__device__ __forceinline__ bool box_contains_pt(const double *mn, const double *mx, D3 p)
{
  return p.x >= __ldg(mn + 0) && p.x <= __ldg(mx + 0) && p.y >= __ldg(mn + 1) && p.y <= __ldg(mx + 1) &&
         p.z >= __ldg(mn + 2) && p.z <= __ldg(mx + 2);
}

// A per-thread array in shared memory, strided by the block size: element i of thread t at
// base[i * stride + t], so the threads of a warp touch consecutive banks.
template <typename T>
struct SArr {
  T *p;
  int stride;
  __device__ __forceinline__ T &operator[](int i) const { return p[i * stride]; }
};

// Traversal scratch of the kernels on the step path (step, multi-job step, walk, locate):
// the BVH stack of the step's traversal, of the relocation's level locate and of point
// location (used one after the other, never nested), then the mixed traversal's candidate
// queue (pv, box-entry lower bound).  It lives in dynamic shared memory, kStepSmemWords words
// per thread strided by the block size, instead of a local-memory stack frame: the frame's
// spills went through L1 to DRAM.  VGN_SMEM_STACK=0 keeps the stacks in local memory.
#ifndef VGN_SMEM_STACK
#define VGN_SMEM_STACK 1
#endif
constexpr int kMaxStepCand   = 16;
constexpr int kStepSmemWords = VGN_SMEM_STACK ? kStackSize + 2 * kMaxStepCand : 0;
// the step's FP64 phase keeps one double per queue slot in the (then free) traversal stack
// and one 4-bit shape type per slot in a 64-bit word
static_assert(2 * kMaxStepCand <= kStackSize && kMaxStepCand <= 16 && kNumShapes <= 16, "step queue layout");
extern __shared__ uint32_t vgn_step_smem[];

#if VGN_SMEM_STACK
#define VGN_TRAVERSAL_STACK(name) \
  const SArr<unsigned> name { vgn_step_smem + threadIdx.x, (int)blockDim.x }
#else
#define VGN_TRAVERSAL_STACK(name) unsigned name[kStackSize]
#endif

// BVH::CheckDaughterIntersections (BVH.h:96-146), FP64
__device__ __forceinline__ bool bvh_check_daughters(const GeomView &g, const LVRec &lv, D3 lp, D3 ld, double &step,
                                                    int last, int &hit)
{
  VGN_TRAVERSAL_STACK(stack);
  int sp        = 1;
  stack[0]      = 0;
  const D3 inv  = d3(1.0 / nonzero(ld.x), 1.0 / nonzero(ld.y), 1.0 / nonzero(ld.z));
  const NodeRec *nodes = g.nodes + lv.nodes_off;
  const PrimRec *prims = g.prims + lv.prims_off;
  do {
    // Inner nodes first: every lane descends until it holds a leaf or its stack runs empty, so
    // that the lanes of a warp reach the leaf code together.  Each lane visits its nodes in the
    // same order as before; only the interleaving across lanes changes.
    unsigned id = 0;
    int nchild  = -1;
    while (sp > 0) {
      id     = stack[--sp];
      nchild = __ldg(&nodes[id].nchild);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      double tminL, tmaxL, tminR, tmaxR;
      slab(nodes[L].mn, nodes[L].mx, lp, inv, tminL, tmaxL);
      slab(nodes[R].mn, nodes[R].mx, lp, inv, tminR, tmaxR);
      const bool trL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < step;
      const bool trR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < step;
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        return false;
      }
      if (tminR < tminL) {
        if (trR) stack[sp++] = R;
        if (trL) stack[sp++] = L;
      } else {
        if (trL) stack[sp++] = L;
        if (trR) stack[sp++] = R;
      }
    }
    if (nchild >= 0) {
      const int off = __ldg(&nodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const PrimRec &q = prims[off + i];
        double tmin, tmax;
        slab(q.mn, q.mx, lp, inv, tmin, tmax);
        if (tmin <= tmax && tmax >= 0.0 && tmin < step) {
          const int vol     = __ldg(&q.pv);
          const double dist = pv_dist_in(g, vol, lp, ld, step);
          if (dist < step && !(dist <= 0.0 && vol == last)) step = dist, hit = vol;
        }
      }
    }
  } while (sp > 0);
  return true;
}

// VUnplacedVolume::ApproachSolid (UnplacedVolume.h:274-281): the ray's entry into the shape's
// bounding box `bb` (min then max corner: its Extent, cached at construction) by
// BoxImplementation::IntersectCachedKernel2 (BoxImplementation.h:326-368), t0 = 0, t1 = kInfLength
__device__ __forceinline__ double approach_solid(const double *bb, D3 p, D3 inv)
{
  const int sx = inv.x < 0, sy = inv.y < 0, sz = inv.z < 0;
  double tmin        = (__ldg(bb + 3 * sx) - p.x) * inv.x;
  const double tymax = (__ldg(bb + 3 * (1 - sy) + 1) - p.y) * inv.y;
  bool done          = tmin > tymax;
  if (done) return kInfLength;
  double tmax        = (__ldg(bb + 3 * (1 - sx)) - p.x) * inv.x;
  const double tymin = (__ldg(bb + 3 * sy + 1) - p.y) * inv.y;
  done |= tymin > tmax;
  if (done) return kInfLength;
  tmin               = vmax(tmin, tymin);
  tmax               = vmin(tmax, tymax);
  const double tzmin = (__ldg(bb + 3 * sz + 2) - p.z) * inv.z;
  const double tzmax = (__ldg(bb + 3 * (1 - sz) + 2) - p.z) * inv.z;
  done |= (tmin > tzmax) || (tzmin > tmax);
  if (done) return kInfLength;
  tmin = vmax(tmin, tzmin);
  tmax = vmin(tmax, tzmax);
  done |= !((tmin <= kInfLength + kTolerance) && (tmax > 0. - kTolerance));
  return done ? kInfLength : tmin;
}

// BVH::ApproachNextDaughter (BVH.cpp:395-449): the traversal of CheckDaughterIntersections with
// each candidate daughter's ApproachSolid, in the daughter's frame, in place of its DistanceToIn
__device__ __forceinline__ bool bvh_approach(const GeomView &g, const LVRec &lv, D3 lp, D3 ld, double &step, int last)
{
  VGN_TRAVERSAL_STACK(stack);
  int sp        = 1;
  stack[0]      = 0;
  const D3 inv  = d3(1.0 / nonzero(ld.x), 1.0 / nonzero(ld.y), 1.0 / nonzero(ld.z));
  const NodeRec *nodes = g.nodes + lv.nodes_off;
  const PrimRec *prims = g.prims + lv.prims_off;
  do {
    const unsigned id = stack[--sp];
    const int nchild  = __ldg(&nodes[id].nchild);
    if (nchild >= 0) {
      const int off = __ldg(&nodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const PrimRec &q = prims[off + i];
        double tmin, tmax;
        slab(q.mn, q.mx, lp, inv, tmin, tmax);
        if (tmin <= tmax && tmax >= 0.0 && tmin < step) {
          const int vol = __ldg(&q.pv);
          PvXf x;
          load_pv_xf(g, vol, x);
          const D3 p        = xf_point(x.t, x.r, lp);
          const D3 d        = xf_dir(x.r, ld);
          const D3 dinv     = d3(1.0 / nonzero(d.x), 1.0 / nonzero(d.y), 1.0 / nonzero(d.z));
          const double dist = approach_solid(g.lv_bbox + 6 * __ldg(&g.pv[vol].lv), p, dinv);
          if (dist < step && !(dist <= 0.0 && vol == last)) step = dist;
        }
      }
    } else {
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      double tminL, tmaxL, tminR, tmaxR;
      slab(nodes[L].mn, nodes[L].mx, lp, inv, tminL, tmaxL);
      slab(nodes[R].mn, nodes[R].mx, lp, inv, tminR, tmaxR);
      const bool trL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < step;
      const bool trR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < step;
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        return false;
      }
      if (tminR < tminL) {
        if (trR) stack[sp++] = R;
        if (trL) stack[sp++] = L;
      } else {
        if (trL) stack[sp++] = L;
        if (trR) stack[sp++] = R;
      }
    }
  } while (sp > 0);
  return true;
}

// BVH::ComputeSafety (BVH.h:172-209), FP64
__device__ __forceinline__ double bvh_safety(const GeomView &g, const LVRec &lv, D3 lp, double safety)
{
  unsigned stack[kStackSize];
  int sp   = 1;
  stack[0] = 0;
  const NodeRec *nodes = g.nodes + lv.nodes_off;
  const PrimRec *prims = g.prims + lv.prims_off;
  do {
    // Inner nodes first: every lane descends until it holds a leaf or its stack runs empty, so
    // that the lanes of a warp reach the leaf code together.  Each lane visits its nodes in the
    // same order as before; only the interleaving across lanes changes.
    unsigned id = 0;
    int nchild  = -1;
    while (sp > 0) {
      id     = stack[--sp];
      nchild = __ldg(&nodes[id].nchild);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      const double sL = box_safety(nodes[L].mn, nodes[L].mx, lp);
      const double sR = box_safety(nodes[R].mn, nodes[R].mx, lp);
      const bool trL = sL < safety, trR = sR < safety;
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        return safety;
      }
      if (sR < sL) {
        if (trR) stack[sp++] = R;
        if (trL) stack[sp++] = L;
      } else {
        if (trL) stack[sp++] = L;
        if (trR) stack[sp++] = R;
      }
    }
    if (nchild >= 0) {
      const int off = __ldg(&nodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const PrimRec &q = prims[off + i];
        if (box_safety(q.mn, q.mx, lp) < safety) {
          const double dist = pv_safe_in(g, __ldg(&q.pv), lp);
          if (dist < safety) safety = dist;
        }
      }
    }
  } while (sp > 0);
  return safety;
}

// BVH::LevelLocate(exclvol, localpoint, pvol, daughterlocalpoint) (BVH.h:255-285)
__device__ __forceinline__ bool bvh_level_locate(const GeomView &g, const LVRec &lv, int excl, D3 lp, int &pvol,
                                                 D3 &dlp)
{
  VGN_TRAVERSAL_STACK(stack);
  int sp   = 1;
  stack[0] = 0;
  const NodeRec *nodes = g.nodes + lv.nodes_off;
  const PrimRec *prims = g.prims + lv.prims_off;
  do {
    // inner nodes first, then the leaf: the lanes of a warp reach the leaf code together
    unsigned id = 0;
    int nchild  = -1;
    while (sp > 0) {
      id     = stack[--sp];
      nchild = __ldg(&nodes[id].nchild);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        return false;
      }
      if (box_contains_pt(nodes[L].mn, nodes[L].mx, lp)) stack[sp++] = L;
      if (box_contains_pt(nodes[R].mn, nodes[R].mx, lp)) stack[sp++] = R;
    }
    if (nchild >= 0) {
      const int off = __ldg(&nodes[id].offset);
      for (int i = 0; i < nchild; ++i) {
        const PrimRec &q = prims[off + i];
        if (box_contains_pt(q.mn, q.mx, lp)) {
          const int vol = __ldg(&q.pv);
          if (vol != excl && pv_contains(g, vol, lp, dlp)) {
            pvol = vol;
            return true;
          }
        }
      }
    }
  } while (sp > 0);
  return false;
}

__device__ __forceinline__ LVRec load_lv(const GeomView &g, int lvi)
{
  LVRec r;
  const int4 *src = reinterpret_cast<const int4 *>(g.lv + lvi);
  int4 a = __ldg(src), b = __ldg(src + 1);
  r.shape = a.x; r.shape_row = a.y; r.nd = a.z; r.daughters_off = a.w;
  r.nodes_off = b.x; r.n_nodes = b.y; r.prims_off = b.z;
  r.depth = (uint16_t)((unsigned)b.w & 0xffffu); r.dtypes = (uint16_t)((unsigned)b.w >> 16);
  return r;
}

__device__ __forceinline__ int pv_lv(const GeomView &g, int pv) { return __ldg(&g.pv[pv].lv); }

}  // namespace VGN_KSET
}  // namespace dev
}  // namespace vgn
