// nav_mixed.cuh -- mixed-precision BVH traversal with results bit-identical
// to the all-FP64 traversal.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, and a BVH
// traversal in one thread per track leaves only a few lanes of each warp
// active at a time.  Two measures keep the FP64 work small and coherent:
//
//  1. Every box test whose only outcome is a decision (visit a node, keep a
//     candidate, which child first) runs in FP32 interval arithmetic with
//     directed rounding (__fsub_rd, __fmul_ru, ...).  The interval provably
//     contains the value the FP64 code would compute, so a decision is known
//     whenever the interval lies on one side of the threshold; otherwise the
//     quantity is recomputed in FP64.
//  2. FP64 shape evaluations are taken out of the divergent traversal loop
//     and run afterwards, where all lanes of a warp execute them together:
//       step   -- the traversal collects the leaf candidates in visit order
//                 (culling may be conservative: a candidate the FP64 code
//                 would have culled lies beyond the step its box test used,
//                 so it can never be accepted); the candidates are then
//                 evaluated in that order with the reference's acceptance
//                 rule.  The child order is always decided exactly, so the
//                 candidate order -- and hence tie-breaking -- is the
//                 reference's.
//       safety -- the reference prunes with the running minimum, so the
//                 pruning decisions must be exact.  Box daughters enter as
//                 FP32-interval contenders; the running minimum is known as
//                 an interval, resolved exactly (FP64) only when a decision
//                 needs it and once at the end.
// Distances that reach the output are always FP64 values computed by the
// same code as the plain kernels.
#pragma once

#include "nav_device.cuh"

namespace vgn {
namespace dev {
inline namespace VGN_KSET {

struct FI {
  float lo, hi;
};

// tri-state decisions
enum : int { kNo = 0, kYes = 1, kMaybe = 2 };

// double -> float rounded toward -inf (up = false) or +inf (up = true), with
// integer operations in the normal float range (the FP64 pipe stays free).
__device__ __forceinline__ float d2f_dir(double x, bool up)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0ull) return (float)x;  // +-0
  const unsigned sign            = (unsigned)(b >> 63);
  const int e                    = (int)((b >> 52) & 0x7ffull);
  const int fe                   = e - 1023 + 127;
  if (e == 0x7ff || fe <= 0 || fe >= 255) return up ? __double2float_ru(x) : __double2float_rd(x);
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  unsigned bits                 = (sign << 31) | ((unsigned)fe << 23) | (unsigned)(mant >> 29);
  const bool inexact            = (mant & 0x1FFFFFFFull) != 0ull;
  if (inexact && (up ? sign == 0u : sign != 0u)) bits += 1u;  // away from zero in the rounding direction
  return __uint_as_float(bits);
}

__device__ __forceinline__ FI fi(double x) { return FI{d2f_dir(x, false), d2f_dir(x, true)}; }
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
// product with a rotation entry's interval: the outward-rounded image of one double, so both
// ends have the double's sign (or are 0) and the interval never contains 0 in its interior
__device__ __forceinline__ FI fi_mul_rot(FI a, FI r) { return fi_mul_signed(a, r, r.hi <= 0.f); }
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
  r.lp   = lp;
  r.ld   = ld;
  r.p[0] = fi(lp.x);
  r.p[1] = fi(lp.y);
  r.p[2] = fi(lp.z);
  const double d[3] = {nonzero(ld.x), nonzero(ld.y), nonzero(ld.z)};  // Global.h:174-178
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const FI di = fi(d[k]);                                  // same sign at both ends: |d| >= 1e-30
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

// Interval of AABB::ComputeIntersectionInvDir's (tmin, tmax) (AABB.h:136-154).
// The FP64 code's swap leaves t(min side) <= t(max side) per axis; which box
// side is "near" only depends on the sign of the inverse direction, by
// monotonicity of rounding.
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

// Interval of max_k(|l_k| - h_k) for a box daughter, l = placement transform
// of the point: BoxImplementation::SafetyToIn (BoxImplementation.h:153-158)
// and the quantity BoxImplementation::Contains compares with 0.
__device__ __forceinline__ FI ibox_safety_in(const IXForm &x, const FI *p)
{
  FI t[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) t[k] = fi_sub(p[k], FI{__ldg(&x.t_lo[k]), __ldg(&x.t_hi[k])});
  FI m;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    FI l = fi_mul_rot(t[0], FI{__ldg(&x.r_lo[i]), __ldg(&x.r_hi[i])});
    l    = fi_add(l, fi_mul_rot(t[1], FI{__ldg(&x.r_lo[3 + i]), __ldg(&x.r_hi[3 + i])}));
    l    = fi_add(l, fi_mul_rot(t[2], FI{__ldg(&x.r_lo[6 + i]), __ldg(&x.r_hi[6 + i])}));
    const FI v = fi_sub(fi_abs(l), FI{__ldg(&x.h_lo[i]), __ldg(&x.h_hi[i])});
    m          = i == 0 ? v : fi_max(m, v);
  }
  return m;
}

// ---- interval SafetyToIn of the other shapes --------------------------------
// Each follows the FP64 operation sequence of the shape's SafetyToIn with outward-
// rounded FP32 intervals over the precomputed enclosures of GeomView::isin, so every
// intermediate interval contains the double the FP64 code computes; a branch the
// intervals cannot decide makes the bound unavailable (false) and the caller falls
// back to FP64.  No FP64 instruction is issued here.
__device__ __forceinline__ FI fi_sqr(FI a)  // a * a
{
  const float l = fabsf(a.lo), h = fabsf(a.hi);
  if (a.lo <= 0.f && a.hi >= 0.f) {
    const float m = fmaxf(l, h);
    return FI{0.f, __fmul_ru(m, m)};
  }
  const float m = fminf(l, h), M = fmaxf(l, h);
  return FI{__fmul_rd(m, m), __fmul_ru(M, M)};
}
__device__ __forceinline__ FI fi_sqrt(FI a) { return FI{__fsqrt_rd(fmaxf(a.lo, 0.f)), __fsqrt_ru(fmaxf(a.hi, 0.f))}; }
__device__ __forceinline__ FI fi_neg(FI a) { return FI{-a.hi, -a.lo}; }
__device__ __forceinline__ FI iq(const float *q, int k)
{
  const float2 v = __ldg(reinterpret_cast<const float2 *>(q) + k);
  return FI{v.x, v.y};
}
__device__ __forceinline__ bool iflag(const float *q, int k) { return __ldg(q + 2 * k) != 0.f; }

// the daughter-frame point: Transformation3D::Transform, (p - t) then the rotation
__device__ __forceinline__ void ixf_local(const IXForm &x, const FI *p, FI *l)
{
  FI t[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) t[k] = fi_sub(p[k], FI{__ldg(&x.t_lo[k]), __ldg(&x.t_hi[k])});
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    FI v = fi_mul_rot(t[0], FI{__ldg(&x.r_lo[i]), __ldg(&x.r_hi[i])});
    v    = fi_add(v, fi_mul_rot(t[1], FI{__ldg(&x.r_lo[3 + i]), __ldg(&x.r_hi[3 + i])}));
    l[i] = fi_add(v, fi_mul_rot(t[2], FI{__ldg(&x.r_lo[6 + i]), __ldg(&x.r_hi[6 + i])}));
  }
}

// TubeImplementation SafetyToInOld (TubeImplementation.h:912-938)
__device__ __forceinline__ bool itube_safe_in(const float *q, const FI *p, FI &out)
{
  FI s       = fi_sub(fi_abs(p[2]), iq(q, irow::TubeZ));
  const FI r = fi_sqrt(fi_add(fi_sqr(p[0]), fi_sqr(p[1])));
  s          = fi_max(s, fi_sub(r, iq(q, irow::TubeRmax)));
  if (iflag(q, irow::TubeHasRmin)) s = fi_max(s, fi_sub(iq(q, irow::TubeRmin), r));
  out = s;
  return true;
}

// ConeImplementation SafetyToIn (ConeImplementation.h:368-432)
__device__ __forceinline__ bool icone_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  const bool hasrmin = iflag(q, ConeHasRmin);
  const FI distz     = fi_sub(fi_abs(p[2]), iq(q, ConeDz));
  const FI rsq       = fi_add(fi_sqr(p[0]), fi_sqr(p[1]));
  int inside         = fi_lt(distz, iq(q, ConeMinusConeTol));
  {  // rsq < |R (R - 2 tol)|, R the outer radius at z (ConeUtilities.h GetRadiusOfConeAtPoint)
    const FI R = iflag(q, ConeOuterConst) ? iq(q, ConeOuterR)
                                          : fi_add(fi_mul_rot(p[2], iq(q, ConeOuterSlope)), iq(q, ConeOuterOffset));
    inside = and3(inside, fi_lt(rsq, fi_abs(fi_mul(R, fi_sub(R, iq(q, ConeTwoOuterTol))))), kYes);
  }
  if (hasrmin) {  // rsq > R (R + 2 tol), R the inner radius at z
    const FI R = iflag(q, ConeInnerConst) ? iq(q, ConeInnerR)
                                          : fi_add(fi_mul_rot(p[2], iq(q, ConeInnerSlope)), iq(q, ConeInnerOffset));
    inside = and3(inside, fi_lt(fi_mul(R, fi_add(R, iq(q, ConeTwoInnerTol))), rsq), kYes);
  }
  if (inside == kMaybe) return false;
  if (inside == kYes) {
    out = FI{-1.f, -1.f};
    return true;
  }
  const FI rho = fi_sqrt(rsq);
  const FI pRMax = fi_add(fi_mul_rot(p[2], iq(q, ConeTanRMax)), iq(q, ConeAvgRmax));
  FI s           = fi_neg(fi_mul_rot(fi_sub(pRMax, rho), iq(q, ConeInvSecRMax)));
  if (hasrmin) {
    const FI pRMin = fi_add(fi_mul_rot(p[2], iq(q, ConeTanRMin)), iq(q, ConeAvgRmin));
    s              = fi_max(s, fi_neg(fi_mul_rot(fi_sub(rho, pRMin), iq(q, ConeInvSecRMin))));
  }
  s = fi_max(distz, s);
  // fabs(safety) < kTolerance ? 0 : safety
  const FI tol = iq(q, ConeTol);
  if (s.lo > -tol.lo && s.hi < tol.lo) {
    s = FI{0.f, 0.f};
  } else if (!(s.lo >= tol.hi || s.hi <= -tol.hi)) {
    return false;
  }
  out = s;
  return true;
}

// TrdUtilities::Safety<inside = false> (TrdImplementation.h:140-168)
__device__ __forceinline__ bool itrd_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  FI dist        = fi_sub(iq(q, TrdDz), fi_abs(p[2]));
  const FI distx = fi_sub(iq(q, TrdHalfX), fi_mul_rot(p[2], iq(q, TrdFx)));
  const int okx  = fi_ge0(distx);
  if (okx == kMaybe) return false;
  if (okx == kYes) dist = fi_min(dist, fi_mul_rot(fi_sub(distx, fi_abs(p[0])), iq(q, TrdCalfX)));
  if (iflag(q, TrdVaryingY)) {
    const FI disty = fi_sub(iq(q, TrdHalfY), fi_mul_rot(p[2], iq(q, TrdFy)));
    const int oky  = fi_ge0(disty);
    if (oky == kMaybe) return false;
    if (oky == kYes) dist = fi_min(dist, fi_mul_rot(fi_sub(disty, fi_abs(p[1])), iq(q, TrdCalfY)));
  } else {
    dist = fi_min(dist, fi_sub(iq(q, TrdDy1), fi_abs(p[1])));
  }
  out = fi_neg(dist);
  return true;
}

// TrapezoidImplementation SafetyToIn over the four side planes (TrapezoidImplementation.h:341-371)
__device__ __forceinline__ bool itrap_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  FI s = fi_sub(fi_abs(p[2]), iq(q, TrapDz));
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    FI d = fi_add(fi_mul_rot(p[0], iq(q, TrapA + i)), fi_mul_rot(p[1], iq(q, TrapB + i)));
    d    = fi_add(fi_add(d, fi_mul_rot(p[2], iq(q, TrapC + i))), iq(q, TrapD + i));
    s    = fi_max(s, d);
  }
  out = s;
  return true;
}

// SphereImplementation SafetyToIn, full sphere (SphereImplementation.h:388-420)
__device__ __forceinline__ bool isphere_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  const bool hasrmin = iflag(q, SphHasRmin);
  const FI rad2      = fi_add(fi_add(fi_sqr(p[0]), fi_sqr(p[1])), fi_sqr(p[2]));
  int cin, cout;
  if (hasrmin) {
    cin         = and3(fi_le(rad2, iq(q, SphMsqMax)), fi_le(iq(q, SphPsqMin), rad2), kYes);
    const int a = fi_le(iq(q, SphPsqMax), rad2), b = fi_le(rad2, iq(q, SphMsqMin));
    cout        = (a == kYes || b == kYes) ? kYes : ((a == kNo && b == kNo) ? kNo : kMaybe);
  } else {
    cin  = fi_le(rad2, iq(q, SphMsqMax));
    cout = fi_le(iq(q, SphPsqMax), rad2);
  }
  if (cin == kMaybe) return false;
  if (cin == kYes) {
    out = FI{-1.f, -1.f};
    return true;
  }
  if (cout == kMaybe) return false;
  if (cout == kNo) {
    out = FI{0.f, 0.f};
    return true;
  }
  const FI rad = fi_sqrt(rad2);
  out = hasrmin ? fi_max(fi_sub(iq(q, SphRmin), rad), fi_sub(rad, iq(q, SphRmax))) : fi_sub(rad, iq(q, SphRmax));
  return true;
}

// OrbImplementation SafetyToIn (OrbImplementation.h:167-177)
__device__ __forceinline__ bool iorb_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  const FI rad = fi_sqrt(fi_add(fi_add(fi_sqr(p[0]), fi_sqr(p[1])), fi_sqr(p[2])));
  const int in = fi_lt(rad, iq(q, OrbRMinusTol));
  if (in == kMaybe) return false;
  if (in == kYes) {
    out = FI{-1.f, -1.f};
    return true;
  }
  const int shell = and3(fi_lt(iq(q, OrbRMinusTol), rad), fi_lt(rad, iq(q, OrbRPlusTol)), kYes);
  if (shell == kMaybe) return false;
  out = shell == kYes ? FI{0.f, 0.f} : fi_sub(rad, iq(q, OrbR));
  return true;
}

// a >= b as a tri-state
__device__ __forceinline__ int fi_ge(FI a, FI b) { return a.lo >= b.hi ? kYes : (a.hi < b.lo ? kNo : kMaybe); }

// PolyconeImplementation SafetyToIn (PolyconeImplementation.h:381-450), full phi: the section
// of the point (PolyconeStruct::GetSectionIndex, PolyconeStruct.h:302-311, decided exactly or
// not at all), its cone's SafetyToIn, and the scan of the neighbouring sections while their
// z distance stays below the running minimum.
__device__ __forceinline__ bool ipcon_safe_in(const float *q, const FI *p, FI &out)
{
  using namespace irow;
  const int n = (int)__ldg(q + 2 * PconN);
  int index   = -2;
  const int below = fi_lt(p[2], iq(q, PconZs));
  if (below == kMaybe) return false;
  if (below == kYes) {
    index = -1;
  } else {
    for (int i = 0; i < n; ++i) {
      const int in = and3(fi_le(iq(q, PconZs + i), p[2]), fi_le(p[2], iq(q, PconZs + i + 1)), kYes);
      if (in == kMaybe) return false;
      if (in == kYes) {
        index = i;
        break;
      }
    }
  }
  const bool needZ = index < 0;
  if (index == -1) index = 0;
  if (index == -2) index = n - 1;
  FI l[3] = {p[0], p[1], fi_sub(p[2], iq(q, pcon_ishift(n) + index))};
  FI s;
  if (!icone_safe_in(q + 2 * pcon_icone(n, index), l, s)) return false;
  if (!needZ) {
    const int small = fi_lt(s, iq(q, PconTol));
    if (small == kMaybe) return false;
    if (small == kNo) {
      FI zbase = iq(q, PconZs + index + 1);
      for (int i = index + 1; i < n; ++i) {
        const int stop = fi_ge(fi_sub(iq(q, PconZs + i), zbase), s);
        if (stop == kMaybe) return false;
        if (stop == kYes) break;
        l[2] = fi_sub(p[2], iq(q, pcon_ishift(n) + i));
        FI si;
        if (!icone_safe_in(q + 2 * pcon_icone(n, i), l, si)) return false;
        s = fi_min(s, si);
      }
      if (index > 0) {
        zbase = iq(q, PconZs + index - 1);
        for (int i = index - 1; i >= 0; --i) {
          const int stop = fi_ge(fi_sub(zbase, iq(q, PconZs + i)), s);
          if (stop == kMaybe) return false;
          if (stop == kYes) break;
          l[2] = fi_sub(p[2], iq(q, pcon_ishift(n) + i));
          FI si;
          if (!icone_safe_in(q + 2 * pcon_icone(n, i), l, si)) return false;
          s = fi_min(s, si);
        }
      }
    }
  }
  out = s;
  return true;
}

// Interval SafetyToIn of a daughter at the mother-frame interval point p: Box from
// IXForm's half-lengths, Tube/Cone/Trd/Trapezoid/Sphere/Orb/Polycone from GeomView::isin;
// false for an undecided branch or a shape without a row (sections, CutTube).
__device__ __forceinline__ bool ishape_safety_in(const GeomView &g, const IXForm &x, const FI *p, FI &out)
{
  const int type = __ldg(&x.shape);
  if (type == kBox) {
    out = ibox_safety_in(x, p);
    return true;
  }
  const int off = __ldg(&x.isin);
  if (off < 0) return false;
  FI l[3];
  ixf_local(x, p, l);
  const float *q = g.isin + 2 * off;
  switch (type) {
  case kTube: return itube_safe_in(q, l, out);
  case kCone: return icone_safe_in(q, l, out);
  case kTrd: return itrd_safe_in(q, l, out);
  case kTrapezoid: return itrap_safe_in(q, l, out);
  case kSphere: return isphere_safe_in(q, l, out);
  case kOrb: return iorb_safe_in(q, l, out);
  case kPolycone: return ipcon_safe_in(q, l, out);
  }
  return false;
}

// ------------------------------------------------------------------ traversal stack entries
// Entries of the mixed traversals' stacks: an internal node is its id; a leaf is its primitive
// range (bit 31, the primitive count in bits 26-29, the first primitive in bits 0-25) when that
// fits, else its id with bits 31 and 30 set (the range is then loaded when it is popped).  A
// child's range is read with the record its box test loads anyway, so visiting an internal node
// costs one dependent load (its children's boxes) instead of two, and a small leaf none.
static_assert(offsetof(INodeSlab, offset) == offsetof(INodeSlab, nchild) + 4 && offsetof(INodeSlab, nchild) % 8 == 0,
              "a node's (nchild, offset) pair is one 8-byte load");
__device__ __forceinline__ int2 inode_range(const INodeSlab *inodes, unsigned id)
{
  return __ldg(reinterpret_cast<const int2 *>(&inodes[id].nchild));
}
__device__ __forceinline__ unsigned stack_entry(unsigned id, int2 range)
{
  if (range.x < 0) return id;
  if (range.x < 16 && (unsigned)range.y < (1u << 26)) return 0x80000000u | ((unsigned)range.x << 26) | (unsigned)range.y;
  return 0xC0000000u | id;
}
// the node of entry e: its id (internal nodes) and its primitive range (nchild < 0: internal)
__device__ __forceinline__ unsigned open_entry(const INodeSlab *inodes, unsigned e, int &nchild, int &off)
{
  nchild = -1;
  off    = 0;
  if (!(e & 0x80000000u)) return e;
  if (!(e & 0x40000000u)) {
    nchild = (int)((e >> 26) & 15u);
    off    = (int)(e & 0x3ffffffu);
    return 0u;
  }
  const unsigned id = e & 0x3fffffffu;
  const int2 range  = inode_range(inodes, id);
  nchild            = range.x;
  off               = range.y;
  return id;
}

// ------------------------------------------------------------------ step
// candidate queue of one track, in visit order (a ring of kMaxStepCand entries)
struct StepCands {
  int n, head;
  uint64_t types;  // shape type of each slot, 4 bits per slot
#if VGN_SMEM_STACK
  SArr<int> pv;
  SArr<float> tmin_lo;
#else
  int pv[kMaxStepCand];
  float tmin_lo[kMaxStepCand];
#endif
  __device__ __forceinline__ int type(int slot) const { return (int)((types >> (4 * slot)) & 0xfull); }
  __device__ __forceinline__ int slot(int k) const { return (head + k) % kMaxStepCand; }
};

// Two 32-bit words per queue slot holding a double: the FP64 DistanceToIn of the slot's
// candidate, computed ahead of the acceptance loop (in the traversal stack, which is free by then).
struct SlotWords {
  unsigned *w;
  int stride;
  __device__ __forceinline__ unsigned &word(int s) const { return w[2 * s * stride]; }
  __device__ __forceinline__ void put(int s, double d) const
  {
    w[2 * s * stride]       = (unsigned)__double2loint(d);
    w[(2 * s + 1) * stride] = (unsigned)__double2hiint(d);
  }
  __device__ __forceinline__ double get(int s) const
  {
    return __hiloint2double((int)w[(2 * s + 1) * stride], (int)w[2 * s * stride]);
  }
};

// Acceptance of one candidate, as in BVH.h:113-118; a candidate whose box is
// entered at or beyond the current step cannot pass dist < step.
__device__ __forceinline__ void eval_step_candidate(const GeomView &g, const MixedRay &r, int pv, float tmin_lo,
                                                    double &step, FI &stepI, int last, int &hit)
{
  if (tmin_lo >= stepI.hi) return;
  const double dist = pv_dist_in(g, pv, r.lp, r.ld, step);
  if (dist < step && !(dist <= 0.0 && pv == last)) {
    step  = dist;
    hit   = pv;
    stepI = fi(step);
  }
}

// BVH::CheckDaughterIntersections (BVH.h:96-146), traversal part: FP32 traversal collecting
// the leaf candidates in visit order into `c` (a candidate is evaluated at once only when
// the queue is full, the oldest first, which keeps the order).
__device__ __forceinline__ bool bvh_collect_step_mixed(const GeomView &g, const LVRec &lv, MixedRay &r,
                                                       double &step, FI &stepI, int last, int &hit, StepCands &c)
{
  VGN_TRAVERSAL_STACK(stack);
  int sp   = 1;
  stack[0] = 0;
  // Culling uses the step after the candidates evaluated so far: never below
  // the step the FP64 traversal would hold at the same point.
  c.n = c.head = 0;
  c.types      = 0;
#if VGN_SMEM_STACK
  c.pv      = SArr<int>{reinterpret_cast<int *>(vgn_step_smem + kStackSize * blockDim.x + threadIdx.x), (int)blockDim.x};
  c.tmin_lo = SArr<float>{reinterpret_cast<float *>(vgn_step_smem + (kStackSize + kMaxStepCand) * blockDim.x + threadIdx.x),
                          (int)blockDim.x};
#endif
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  stack[0]                = stack_entry(0u, inode_range(inodes, 0u));
  bool ok = true;
  do {
    // Inner nodes first: every lane descends until it holds a leaf or its stack runs empty, so
    // that the lanes of a warp reach the leaf code together.  Each lane visits its nodes in the
    // same order as before; only the interleaving across lanes changes.
    int nchild = -1, off = 0;
    unsigned id = 0;
    while (sp > 0) {
      id = open_entry(inodes, stack[--sp], nchild, off);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      const unsigned eL = stack_entry(L, inode_range(inodes, L)), eR = stack_entry(R, inode_range(inodes, R));
      FI tminL, tmaxL, tminR, tmaxR;
      islab(inodes[L].mn_lo, inodes[L].mn_hi, inodes[L].mx_lo, inodes[L].mx_hi, r, tminL, tmaxL);
      islab(inodes[R].mn_lo, inodes[R].mn_hi, inodes[R].mx_lo, inodes[R].mx_hi, r, tminR, tmaxR);
      const bool trL = slab_decision(tminL, tmaxL, stepI) != kNo;
      const bool trR = slab_decision(tminR, tmaxR, stepI) != kNo;
      int rfirst     = kNo;
      if (trL && trR) {
        rfirst = fi_lt(tminR, tminL);
        if (rfirst == kMaybe) {  // the visit order must be the reference's: decide in FP64
          const D3 inv = ray_inv64(r);
          double a, b, cc, d;
          slab(nodes[L].mn, nodes[L].mx, r.lp, inv, a, b);
          slab(nodes[R].mn, nodes[R].mx, r.lp, inv, cc, d);
          rfirst = cc < a ? kYes : kNo;
        }
      }
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        ok = false;
        break;
      }
      if (rfirst == kYes) {
        if (trR) stack[sp++] = eR;
        if (trL) stack[sp++] = eL;
      } else {
        if (trL) stack[sp++] = eL;
        if (trR) stack[sp++] = eR;
      }
    }
    if (!ok) break;
    if (nchild >= 0) {
      for (int i = 0; i < nchild; ++i) {
        const IPrimSlab &q = iprims[off + i];
        FI tmin, tmax;
        islab(q.mn_lo, q.mn_hi, q.mx_lo, q.mx_hi, r, tmin, tmax);
        if (slab_decision(tmin, tmax, stepI) == kNo) continue;
        if (c.n == kMaxStepCand) {  // full: evaluate the oldest now (keeps the order)
          eval_step_candidate(g, r, c.pv[c.head], c.tmin_lo[c.head], step, stepI, last, hit);
          c.head = (c.head + 1) % kMaxStepCand;
          --c.n;
        }
        const int slot   = (c.head + c.n) % kMaxStepCand;
        c.pv[slot]       = __ldg(&q.pv);
        c.tmin_lo[slot]  = tmin.lo;
        c.types = (c.types & ~(0xfull << (4 * slot))) | ((uint64_t)__ldg(&q.shape) << (4 * slot));
        ++c.n;
      }
    }
  } while (sp > 0);
  return ok;
}

// Slots whose DistanceToIn may be computed ahead of the acceptance loop: every candidate
// but the cut tubes (their DistanceToIn takes the running step) whose box entry lies below
// the current step.  The step only decreases, so the acceptance loop reaches no other slot
// but cut tubes.  `present` receives the shape types of those slots.
__device__ __forceinline__ unsigned step_pending(const StepCands &c, FI stepI, unsigned &present)
{
  unsigned done = 0;
  present       = 0;
  for (int k = 0; k < c.n; ++k) {
    const int slot = c.slot(k);
    const int t    = c.type(slot);
    if (c.tmin_lo[slot] >= stepI.hi || t == kCutTube) continue;
    done |= 1u << slot;
    present |= 1u << t;
  }
  return done;
}

// The reference's acceptance rule over the queue in visit order, with the distances of the
// `done` slots read from `sw`; cut tubes are evaluated here with the running step.
__device__ __forceinline__ void step_replay(const GeomView &g, const MixedRay &r, const StepCands &c, unsigned done,
                                            SlotWords sw, double &step, FI &stepI, int last, int &hit)
{
  for (int k = 0; k < c.n; ++k) {
    const int slot = c.slot(k);
    if (c.tmin_lo[slot] >= stepI.hi) continue;
    const int pv      = c.pv[slot];
    const double dist = ((done >> slot) & 1u) ? sw.get(slot) : pv_dist_in(g, pv, r.lp, r.ld, step);
    if (dist < step && !(dist <= 0.0 && pv == last)) {
      step  = dist;
      hit   = pv;
      stepI = fi(step);
    }
  }
}

// BVH::CheckDaughterIntersections (BVH.h:96-146): FP32 traversal collecting candidates in
// visit order, then FP64 evaluation in that order.
__device__ __forceinline__ bool bvh_check_daughters_mixed(const GeomView &g, const LVRec &lv, MixedRay &r,
                                                          double &step, int last, int &hit)
{
  FI stepI = fi(step);
  StepCands c;
  const bool ok = bvh_collect_step_mixed(g, lv, r, step, stepI, last, hit, c);
  // FP64 phase.  Daughters of one shape type: the candidates in visit order with the
  // reference's acceptance rule, the lanes of a warp running the same shape code.
  if ((lv.dtypes & (lv.dtypes - 1)) == 0) {
    for (int k = 0; k < c.n; ++k) {
      const int slot = c.slot(k);
      eval_step_candidate(g, r, c.pv[slot], c.tmin_lo[slot], step, stepI, last, hit);
    }
    return ok;
  }
  // Several types.  A candidate's DistanceToIn does not depend on when it is computed (the
  // cut tube's excepted), so the values are computed first, grouped by shape type -- the
  // lanes of a warp run one shape's code at a time, each on its own candidates of that
  // type, instead of every lane its own shape -- and the acceptance rule then runs over them.
#if VGN_SMEM_STACK
  const SlotWords sw{vgn_step_smem + threadIdx.x, (int)blockDim.x};
#else
  unsigned words[2 * kMaxStepCand];
  const SlotWords sw{words, 1};
#endif
  unsigned present;
  const unsigned done = step_pending(c, stepI, present);
  for (int t = 0; t < kNumShapes; ++t) {
    if (!((present >> t) & 1u)) continue;
    unsigned m = 0;
    for (unsigned rest = done; rest; rest &= rest - 1) {
      const int s = __ffs(rest) - 1;
      if (c.type(s) == t) m |= 1u << s;
    }
    while (m) {
      const int s = __ffs(m) - 1;
      m &= m - 1;
      sw.put(s, pv_dist_in(g, c.pv[s], r.lp, r.ld, kInfLength));
    }
  }
  step_replay(g, r, c, done, sw, step, stepI, last, hit);
  return ok;
}

// ------------------------------------------------------------------ safety
constexpr int kMaxSafeCand = 8;

// Running minimum of BVH::ComputeSafety known as: an exact part `known`
// (mother safety and daughters evaluated in FP64) and pending daughters whose
// SafetyToIn is known as an FP32 interval (ishape_safety_in).
struct SafeRun {
  double known;
  FI knownI;
  int n;
  SArr<int> pv;  // kMaxSafeCand pending daughters, in shared memory
  SArr<float> lo, hi;
  FI cur;  // interval of the current running minimum
};

// Dynamic shared memory of the kernels that run bvh_safety_mixed: per thread the traversal
// stack and the pending daughters, kSafetySmemWords words strided by the block size.
constexpr int kSafetySmemWords = kStackSize + 3 * kMaxSafeCand;
extern __shared__ uint32_t vgn_safety_smem[];

__device__ __forceinline__ void saferun_update(SafeRun &s)
{
  FI c = s.knownI;
  for (int k = 0; k < s.n; ++k) c = FI{fminf(c.lo, s.lo[k]), fminf(c.hi, s.hi[k])};
  s.cur = c;
}

// evaluate all pending daughters in FP64: the running minimum becomes exact
__device__ __forceinline__ void saferun_resolve(const GeomView &g, const MixedRay &r, SafeRun &s)
{
  for (int k = 0; k < s.n; ++k) {
    if (s.lo[k] >= s.cur.hi) continue;  // cannot be the minimum
    const double d = pv_safe_in(g, s.pv[k], r.lp);
    if (d < s.known) s.known = d;
  }
  s.n      = 0;
  s.knownI = fi(s.known);
  s.cur    = s.knownI;
}

// decision x < (running minimum), resolving the minimum when the intervals overlap;
// `exact` is the FP64 value of x (computed only if still needed)
template <typename ExactFn>
__device__ __forceinline__ bool saferun_less(const GeomView &g, const MixedRay &r, SafeRun &s, FI x, ExactFn exact)
{
  int dec = fi_lt(x, s.cur);
  if (dec != kMaybe) return dec == kYes;
  if (s.n > 0) {
    saferun_resolve(g, r, s);
    dec = fi_lt(x, s.cur);
    if (dec != kMaybe) return dec == kYes;
  }
  return exact() < s.known;
}

// BVH::ComputeSafety (BVH.h:172-209) with exact pruning decisions and deferred
// FP64 evaluation of the daughters that have an interval SafetyToIn (all shapes
// but Polycone, which is evaluated in FP64 at once).
__device__ __forceinline__ double bvh_safety_mixed(const GeomView &g, const LVRec &lv, const MixedRay &r,
                                                   double safety)
{
  const int stride = blockDim.x;
  uint32_t *base   = vgn_safety_smem + threadIdx.x;
  const SArr<unsigned> stack{base, stride};
  int sp = 1;
  SafeRun s;
  s.pv     = SArr<int>{reinterpret_cast<int *>(base + kStackSize * stride), stride};
  s.lo     = SArr<float>{reinterpret_cast<float *>(base + (kStackSize + kMaxSafeCand) * stride), stride};
  s.hi     = SArr<float>{reinterpret_cast<float *>(base + (kStackSize + 2 * kMaxSafeCand) * stride), stride};
  s.known  = safety;
  s.knownI = fi(safety);
  s.n      = 0;
  s.cur    = s.knownI;
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const ISafe *isafe_n    = g.inode_safe + lv.nodes_off;
  const ISafe *isafe_p    = g.iprim_safe + lv.prims_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  const PrimRec *prims    = g.prims + lv.prims_off;
  stack[0]                = stack_entry(0u, inode_range(inodes, 0u));
  bool ok                 = true;
  do {
    // Inner nodes first: every lane descends until it holds a leaf or its stack runs empty,
    // so that the lanes of a warp reach the leaf code (the costly part) together.  Each lane
    // visits its nodes in the same order as before; only the interleaving across lanes changes.
    int nchild = -1, off = 0;
    while (sp > 0) {
      const unsigned id = open_entry(inodes, stack[--sp], nchild, off);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      const unsigned eL = stack_entry(L, inode_range(inodes, L)), eR = stack_entry(R, inode_range(inodes, R));
      const FI sL = isafety(isafe_n[L], r);
      const FI sR = isafety(isafe_n[R], r);
      const bool trL = saferun_less(g, r, s, sL, [&] { return box_safety(nodes[L].mn, nodes[L].mx, r.lp); });
      const bool trR = saferun_less(g, r, s, sR, [&] { return box_safety(nodes[R].mn, nodes[R].mx, r.lp); });
      bool rfirst    = false;
      if (trL && trR) {
        const int o = fi_lt(sR, sL);
        rfirst = o == kMaybe ? box_safety(nodes[R].mn, nodes[R].mx, r.lp) < box_safety(nodes[L].mn, nodes[L].mx, r.lp)
                             : o == kYes;
      }
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        ok = false;
        break;
      }
      if (rfirst) {
        if (trR) stack[sp++] = eR;
        if (trL) stack[sp++] = eL;
      } else {
        if (trL) stack[sp++] = eL;
        if (trR) stack[sp++] = eR;
      }
    }
    if (!ok) break;
    if (nchild >= 0) {
      for (int i = 0; i < nchild; ++i) {
        // cheapest test first: the primitive's box safety against the running minimum
        const FI sbox = isafety(isafe_p[off + i], r);
        const int pre = fi_lt(sbox, s.cur);
        if (pre == kNo) continue;
        const int vol   = __ldg(&iprims[off + i].pv);
        const IXForm &x = g.ixf[vol];
        FI d{0.f, 0.f};
        const bool bound = ishape_safety_in(g, x, r.p, d);
        if (bound && d.lo >= s.cur.hi) continue;  // SafetyToIn >= running minimum: no update either way
        const PrimRec &pr = prims[off + i];
        if (pre == kMaybe && !saferun_less(g, r, s, sbox, [&] { return box_safety(pr.mn, pr.mx, r.lp); })) continue;
        if (bound) {
          if (s.n == kMaxSafeCand) saferun_resolve(g, r, s);
          s.pv[s.n] = vol;
          s.lo[s.n] = d.lo;
          s.hi[s.n] = d.hi;
          ++s.n;
          saferun_update(s);
        } else {
          const double dist = pv_safe_in(g, vol, r.lp);
          if (dist < s.known) {
            s.known  = dist;
            s.knownI = fi(dist);
          }
          saferun_update(s);
        }
      }
    }
  } while (sp > 0);
  if (s.n > 0) saferun_resolve(g, r, s);  // FP64 phase, coherent across the warp
  return s.known;
}

// ------------------------------------------------------------------ locate
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
  VGN_TRAVERSAL_STACK(stack);
  int sp = 1;
  const FI p[3] = {fi(lp.x), fi(lp.y), fi(lp.z)};
  const INodeSlab *inodes = g.inodes + lv.nodes_off;
  const IPrimSlab *iprims = g.iprims + lv.prims_off;
  const NodeRec *nodes    = g.nodes + lv.nodes_off;
  const PrimRec *prims    = g.prims + lv.prims_off;
  stack[0]                = stack_entry(0u, inode_range(inodes, 0u));
  do {
    // inner nodes first, then the leaf: the lanes of a warp reach the leaf code together
    int nchild = -1, off = 0;
    while (sp > 0) {
      const unsigned id = open_entry(inodes, stack[--sp], nchild, off);
      if (nchild >= 0) break;
      const unsigned L = 2 * id + 1, R = 2 * id + 2;
      if (sp + 2 > g.stack_limit) {
        raise_error(g, kErrStack);
        return false;
      }
      int cL = icontains(inodes[L].mn_lo, inodes[L].mn_hi, inodes[L].mx_lo, inodes[L].mx_hi, p);
      if (cL == kMaybe) cL = box_contains_pt(nodes[L].mn, nodes[L].mx, lp) ? kYes : kNo;
      if (cL == kYes) stack[sp++] = stack_entry(L, inode_range(inodes, L));
      int cR = icontains(inodes[R].mn_lo, inodes[R].mn_hi, inodes[R].mx_lo, inodes[R].mx_hi, p);
      if (cR == kMaybe) cR = box_contains_pt(nodes[R].mn, nodes[R].mx, lp) ? kYes : kNo;
      if (cR == kYes) stack[sp++] = stack_entry(R, inode_range(inodes, R));
    }
    if (nchild >= 0) {
      for (int i = 0; i < nchild; ++i) {
        const IPrimSlab &q = iprims[off + i];
        int dec = icontains(q.mn_lo, q.mn_hi, q.mx_lo, q.mx_hi, p);
        if (dec == kMaybe) dec = box_contains_pt(prims[off + i].mn, prims[off + i].mx, lp) ? kYes : kNo;
        if (dec != kYes) continue;
        const int vol = __ldg(&q.pv);
        if (vol == excl) continue;
        const IXForm &x = g.ixf[vol];
        // a box daughter surely not containing the point needs no FP64 test
        if (__ldg(&x.shape) == kBox && fi_ge0(ibox_safety_in(x, p)) == kYes) continue;
        if (pv_contains(g, vol, lp, dlp)) {
          pvol = vol;
          return true;
        }
      }
    }
  } while (sp > 0);
  return false;
}

}  // namespace VGN_KSET
}  // namespace dev
}  // namespace vgn
