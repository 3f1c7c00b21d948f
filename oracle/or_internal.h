/*
 * or_internal.h -- internal types of the CPU oracle (test infrastructure only).
 * Restates the scalar semantics of VecGeom 1.2.0 base types:
 *   Vector3D      VecGeom/base/Vector3D.h
 *   Transformation3D VecGeom/base/Transformation3D.h:59-63, 561-1000
 *   AABB          VecGeom/base/AABB.h:26-228
 *   constants     VecGeom/base/Math.h:26-53, VecGeom/base/Global.h:142-178
 * The VecCore scalar calls the reference uses are restated as:
 *   Min(a,b) = a < b ? a : b,  Max(a,b) = a > b ? a : b,  Sign(x) = copysign(1,x),
 *   MaskedAssign(d,m,v) = if (m) d = v,  Blend(m,a,b) = m ? a : b.
 */
#ifndef OR_INTERNAL_H
#define OR_INTERNAL_H

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "vgoracle.h"

/* Math.h:27-53 (double precision branch) */
#define kTolerance 1e-9
#define kHalfTolerance (0.5 * kTolerance)
#define kPushTolerance 1e-6
#define kConeTolerance 1e-7
#define kInfLength DBL_MAX
#define kEpsilon DBL_EPSILON
#define kTiny 1e-30
#define kPi 3.14159265358979323846
#define kTwoPi (2. * kPi)
#define kHalfPi (0.5 * kPi)
#define kAngTolerance 1e-9
#define kSqrtTolerance 3.1622777e-5 /* base/Math.h:29 */

typedef struct { double x, y, z; } v3;

static inline v3 v3_make(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 v3_add(v3 a, v3 b) { return v3_make(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v3_sub(v3 a, v3 b) { return v3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v3_mul(v3 a, v3 b) { return v3_make(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 v3_scale(double s, v3 a) { return v3_make(s * a.x, s * a.y, s * a.z); }
static inline v3 v3_abs(v3 a) { return v3_make(fabs(a.x), fabs(a.y), fabs(a.z)); }
static inline double or_min(double a, double b) { return a < b ? a : b; }
static inline double or_max(double a, double b) { return a > b ? a : b; }
/* vecCore::math::Min/Max of three, as used by Vector3D::Min/Max (Vector3D.h:276-280) */
static inline double v3_minc(v3 a) { return or_min(or_min(a.x, a.y), a.z); }
static inline double v3_maxc(v3 a) { return or_max(or_max(a.x, a.y), a.z); }
static inline double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double v3_mag2(v3 a) { return v3_dot(a, a); }
static inline double v3_perp2(v3 a) { return a.x * a.x + a.y * a.y; }
static inline double or_sign(double x) { return copysign(1.0, x); }
/* Global.h:166-178 */
static inline double NonZeroAbs(double x) { return fabs(x) + 1.0e-30; }
static inline double NonZero(double x) { return x + copysign(1.0e-30, x); }

/* Transformation3D members (Transformation3D.h:59-63) */
typedef struct {
  double t[3];
  double r[9];
  int identity, has_rot, has_trans;
} or_xf;

void xf_identity(or_xf *m);
void xf_from12(or_xf *m, const double *a12);           /* 12-parameter constructor + SetProperties */
v3 xf_transform(const or_xf *m, v3 p);                   /* Transform<kGeneric,kGeneric> */
v3 xf_transform_dir(const or_xf *m, v3 d);               /* TransformDirection<kGeneric> */
v3 xf_inverse_transform(const or_xf *m, v3 p);           /* InverseTransform */
void xf_multiply_from_right(or_xf *m, const or_xf *rhs); /* MultiplyFromRight */

/* AABB (AABB.h) */
typedef struct { v3 mn, mx; } or_aabb;
void aabb_intersect_invdir(const or_aabb *b, v3 p, v3 invdir, double *tmin, double *tmax);
static inline double aabb_safety(const or_aabb *b, v3 p)
{
  /* AABB.h:81: ((point - Center()).Abs() - 0.5 * Size()).Max() */
  v3 c = v3_scale(0.5, v3_add(b->mx, b->mn));
  v3 s = v3_sub(b->mx, b->mn);
  return v3_maxc(v3_sub(v3_abs(v3_sub(p, c)), v3_scale(0.5, s)));
}
static inline int aabb_contains(const or_aabb *b, v3 p)
{
  return p.x >= b->mn.x && p.x <= b->mx.x && p.y >= b->mn.y && p.y <= b->mx.y && p.z >= b->mn.z && p.z <= b->mx.z;
}

/* ---- shape parameter structs (cached members as the reference's *Struct) ---- */
typedef struct { double d[3]; } or_box; /* BoxStruct.h fDimensions */

typedef struct { /* evolution::Wedge (Wedge_Evolution.h:43-50), source/Wedge_Evolution.cpp:17-99 */
  double a1x, a1y, a2x, a2y; /* fAlongVector1/2 */
  double n1x, n1y, n2x, n2y; /* fNormalVector1/2 */
  double dphi;               /* fDPhi */
} or_wedge;

typedef struct { /* TubeStruct.h:15-41 */
  double rmin, rmax, z, sphi, dphi;
  double rmin2, rmax2, alongphi1x, alongphi1y, alongphi2x, alongphi2y;
  double tolIrmin2, tolOrmin2, tolIrmax2, tolOrmax2, tolIz, tolOz, tolIrmin, tolOrmin, tolIrmax, tolOrmax, maxval;
  or_wedge w; /* fPhiWedge, built from the constructor's raw (dphi, sphi) */
} or_tube;

typedef struct { /* ConeStruct.h:23-77 cached members */
  double rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi;
  double o_rmin1, o_rmin2, o_rmax1, o_rmax2; /* _frmin1.. (constructor arguments) */
  double innerSlope, outerSlope, innerOffset, outerOffset, innerTolerance, outerTolerance;
  double sqRmin1, sqRmin2, sqRmax1, sqRmax2, tolIz, tolOz;
  double innerConeApex, tanInnerApexAngle, outerConeApex, tanOuterApexAngle;
  double secRMin, secRMax, invSecRMin, invSecRMax, tanRMin, tanRMax, zNormInner, zNormOuter;
  double originalRmax1, originalRmax2;
  double alongphi1x, alongphi1y, alongphi2x, alongphi2y; /* from the checked (sphi, dphi) */
  or_wedge w; /* fPhiWedge: vectors from the raw constructor angles, fDPhi the checked one */
} or_cone;

typedef struct { /* TrdStruct.h:19-39 (UniversalTrd: VECGEOM_NO_SPECIALIZATION is the default build) */
  double dx1, dx2, dy1, dy2, dz;
  double x2minusx1, y2minusy1, halfx1plusx2, halfy1plusy2, calfx, calfy, secxz, secyz, tolx, toly, fx, fy;
} or_trd;

typedef struct { /* TrapezoidStruct.h:41-59 with the PlaneShell<4> side planes (VECGEOM_PLANESHELL=ON) */
  double dz, theta, phi, dy1, dx1, dx2, tanAlpha1, dy2, dx3, dx4, tanAlpha2;
  double tthetaCphi, tthetaSphi;
  double a[4], b[4], c[4], d[4];
} or_trap;

typedef struct { /* ThetaCone (ThetaCone_Evolution.h:45-83) */
  double sT, dT, eT;             /* fSTheta, fDTheta, fETheta */
  double tanS, tanE, tanS2, tanE2; /* tanSTheta, tanETheta and their squares */
  double tanBis, slope1, slope2; /* tanBisector, slope1, slope2 */
} or_theta;

typedef struct { /* SphereStruct.h:21-51 */
  double rmin, rmax;
  double sPhi, dPhi;             /* checked fSPhi, fDPhi (CheckPhiAngles) */
  double sTheta, dTheta, eTheta; /* fSTheta, checked fDTheta (CheckThetaAngles), eTheta */
  int fullPhi, fullTheta, full;  /* fFullPhiSphere, fFullThetaSphere, fFullSphere */
  or_wedge w;  /* evolution::Wedge built from the constructor's raw (dphi, sphi) */
  or_theta tc; /* ThetaCone built from the constructor's raw (stheta, dtheta) */
} or_sphere;

typedef struct { /* PolyconeStruct.h:24-37: z planes and one ConeStruct per section */
  int nsec;
  double startPhi, deltaPhi; /* fStartPhi, fDeltaPhi after PolyconeStruct::Init */
  double *zs;    /* [nsec + 1] fZs */
  double *shift; /* [nsec] PolyconeSection::fShift */
  or_cone *sec;  /* [nsec] PolyconeSection::fSolid */
} or_polycone;

typedef struct { double r; } or_orb; /* OrbStruct.h:19 fR */

typedef struct { /* Plane (VecGeom/volumes/Plane.h:22-95): unit normal and signed distance */
  double n[3], d;
} or_plane;

typedef struct { /* CutTubeStruct.h:21-46 */
  double dz;            /* fDz */
  or_tube tube;         /* fTubeStruct: the tube with an infinite half-length */
  or_plane cut[2];      /* fCutPlanes: bottom, top */
  double cosphi1, sinphi1, cosphi2, sinphi2, maxval;
} or_cuttube;

typedef struct { /* one face of Quadrilaterals (Quadrilaterals.h:25-36) */
  double n[3], d;         /* fPlanes: unit normal and distance */
  double sn[4][3], sd[4]; /* fSideVectors[j]: the side planes */
  double c[4][3];         /* fCorners[j] */
} or_quad;

typedef struct { int n; or_quad *q; } or_quads;

typedef struct { or_quads outer, phi, inner; } or_zseg; /* ZSegment (PolyhedronStruct.h:36-46) */

typedef struct { /* PolyhedronStruct.h:52-80 */
  int sides, nz;                       /* fSideCount, fZPlanes.size() */
  int hasInner, hasPhi, hasLargePhi;   /* fHasInnerRadii, fHasPhiCutout, fHasLargePhiCutout */
  double phiStart, phiDelta;           /* fPhiStart (normalised), fPhiDelta (at most 2 pi) */
  or_wedge w;                          /* fPhiWedge(fPhiDelta, fPhiStart) */
  or_zseg *seg;                        /* [nz - 1] fZSegments */
  double *z, *rmin, *rmax;             /* [nz] fZPlanes, fRMin, fRMax */
  int *samez;                          /* [nz] fSameZ */
  v3 *phisec;                          /* [sides + 1] fPhiSections */
  or_tube btube;                       /* fBoundingTube */
  double btubeOffset;                  /* fBoundingTubeOffset */
} or_polyhedron;

typedef struct { /* TorusStruct2.h:22-32 */
  double rmin, rmax, rtor, sphi, dphi, rmin2, rmax2, rtor2;
  or_wedge w;     /* fPhiWedge(dphi, sphi) */
  or_tube btube;  /* fBoundingTube */
} or_torus;

struct or_lv_s;
typedef struct { /* BooleanStruct (BooleanStruct.h:23-25): the operation and the two placed operands */
  int op;                             /* 0 union, 1 intersection, 2 subtraction (BooleanStruct.h:9) */
  int left_pv, right_pv;              /* the operand placements (pv_mother OR_BOOLEAN_OPERAND) */
  const struct or_lv_s *left, *right; /* their logical volumes */
  or_xf lxf, rxf;                     /* their placements' transformations */
} or_boolean;

typedef struct or_lv_s {
  int type;
  int param_off;
  int nd;           /* number of daughters */
  int *daughters;   /* placed-volume ids, in placement order */
  /* shape */
  union {
    or_box box;
    or_tube tube;
    or_cone cone;
    or_trd trd;
    or_trap trap;
    or_sphere sph;
    or_polycone pcon;
    or_orb orb;
    or_cuttube ctube;
    or_boolean boo;
    or_polyhedron phd;
    or_torus tor;
  } s;
  v3 bbox_min, bbox_max; /* VUnplacedVolume::fBBox: the shape's Extent (UnplacedVolume.h:45, 76-80) */
  /* BVH (BVH.h:364-370), present when nd > 0 */
  int bvh_depth, bvh_nodes;
  int *prim_id, *offset, *nchild;
  or_aabb *nodes, *aabbs;
} or_lv;

typedef struct {
  int lv;
  int mother_lv;
  int child_id;
  or_xf xf;
} or_pv;

struct or_geom {
  int n_lv, n_pv, world_pv;
  or_lv *lv;
  or_pv *pv;
  uint32_t *navind;
  size_t navind_words;
  int max_depth;
  int cache_depth; /* GeoManager::SetTransformationCacheDepth; 0 = every level cached */
};

/* shapes (or_shapes.c) */
int shape_init(or_lv *lv, const double *p, int n_params_avail, char *err, int errlen);
void shape_extent(const or_lv *lv, v3 *mn, v3 *mx);
double shape_dist_in(const or_lv *lv, v3 p, v3 d, double stepmax, or_counters *c);
double shape_dist_out(const or_lv *lv, v3 p, v3 d, double stepmax, or_counters *c);
double shape_safe_in(const or_lv *lv, v3 p, or_counters *c);
double shape_safe_out(const or_lv *lv, v3 p, or_counters *c);
int shape_contains(const or_lv *lv, v3 p, or_counters *c);
void polyhedron_free(or_polyhedron *t);
int shape_inside(const or_lv *lv, v3 p, or_counters *c); /* EInside: kInside=1, kSurface=2, kOutside=3 */

/* BVH build (or_bvh.c) */
int bvh_build(or_geom *g, int lv);

#endif
