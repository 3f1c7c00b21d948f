// geom_types.h -- device-resident geometry layout shared by the host builder
// and the CUDA kernels.
//
// Everything the navigation kernels read lives in a handful of flat,
// read-only arrays that stay resident in HBM (and, being a few MiB at most,
// in the 129 MB L2):
//   navind    the navigation index table, byte-for-byte the reference layout
//             (source/NavIndexTable.cpp:9-99) so NavStateIndex values match
//   pv        one 128-byte record per placed volume (transform + ids)
//   lv        one 32-byte record per logical volume
//   nodes     BVH nodes, 64-byte records, complete binary tree per volume
//   prims     leaf primitives (daughter AABB + placed-volume id) stored in BVH
//             leaf order, so a leaf's candidates are one contiguous run
//   fnodes/fprims  the same boxes rounded outward to FP32 (mixed precision)
//   shape     per-volume shape parameter rows (doubles, cached members)
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define VGN_HD __host__ __device__
#else
#define VGN_HD
#endif

namespace vgn {

constexpr int kStackSize = 32;  // BVH::BVH_MAX_DEPTH (BVH.h:33)
constexpr int kMaxLevels = 30;  // bound on geometry depth (relocation loops)

enum ShapeType : int32_t {
  kBox = 0, kTube = 1, kCone = 2, kTrd = 3, kTrapezoid = 4, kSphere = 5, kPolycone = 6, kOrb = 7, kCutTube = 8,
  kBoolean = 9, kPolyhedron = 10, kTorus = 11, kNumShapes = 12
};

// flags of a placement transformation (Transformation3D::SetProperties,
// source/Transformation3D.cpp:117-126); none set = identity
enum XfFlags : int32_t { kXfTrans = 1, kXfRot = 2 };

// device error bits (OR-ed into the status word)
enum DevError : uint32_t { kErrStack = 1u, kErrRelocate = 2u, kErrState = 4u };

struct alignas(16) XForm {
  double t[3];  // Transformation3D::fTranslation
  double r[9];  // Transformation3D::fRotation (row-major as in the reference)
};

struct alignas(128) PVRec {
  XForm xf;           // placement transformation (mother frame -> this volume's frame)
  int32_t lv;         // logical volume placed
  int32_t child_id;   // position in the mother's daughter list
  int32_t shape;      // shape type of lv (cached)
  int32_t shape_row;  // offset of lv's shape row in GeomView::shape (cached)
  int32_t xf_flags;   // kXfTrans | kXfRot: Transformation3D::HasTranslation / HasRotation of xf
  int32_t pad[3];
};
static_assert(sizeof(PVRec) == 128, "PVRec must be 128 bytes");

struct alignas(32) LVRec {
  int32_t shape;
  int32_t shape_row;
  int32_t nd;            // number of daughters
  int32_t daughters_off; // into GeomView::daughters
  int32_t nodes_off;     // first BVH node (into nodes / fnodes)
  int32_t n_nodes;       // (2 << depth) - 1, 0 if no daughters
  int32_t prims_off;     // first leaf primitive (into prims / fprims)
  uint16_t depth;        // BVH depth
  uint16_t dtypes;       // bit t set: some daughter is of ShapeType t
};
static_assert(sizeof(LVRec) == 32, "LVRec must be 32 bytes");

struct alignas(64) NodeRec {
  double mn[3], mx[3];
  int32_t nchild;  // -1 internal, >= 0 leaf (BVH.cpp:85-86)
  int32_t offset;  // first primitive position of this node
  int32_t pad[2];
};
static_assert(sizeof(NodeRec) == 64, "NodeRec must be 64 bytes");

struct alignas(64) PrimRec {
  double mn[3], mx[3];  // daughter AABB with the 1e-3 margin (ABBoxManager.cpp:141-142)
  int32_t pv;           // placed volume id
  int32_t prim;         // daughter index in the mother
  int32_t pad[2];
};
static_assert(sizeof(PrimRec) == 64, "PrimRec must be 64 bytes");

// FP32 boxes rounded outward (min toward -inf, max toward +inf): a superset of
// the FP64 box, so a conservative FP32 slab test never drops a candidate.
struct alignas(32) FNodeRec {
  float mn[3], mx[3];
  int32_t nchild;
  int32_t offset;
};
static_assert(sizeof(FNodeRec) == 32, "FNodeRec must be 32 bytes");

struct alignas(32) FPrimRec {
  float mn[3], mx[3];
  int32_t pv;
  int32_t prim;
};
static_assert(sizeof(FPrimRec) == 32, "FPrimRec must be 32 bytes");

// ---- FP32 interval images for the mixed-precision kernels ----
// Every float pair [lo, hi] brackets a double of the FP64 tables (lo rounded
// toward -inf, hi toward +inf), so FP32 interval arithmetic with directed
// rounding bounds the value the FP64 code would compute; a decision is taken
// in FP32 only when the whole interval falls on one side.
struct alignas(64) INodeSlab {  // BVH node box, for slab tests
  float mn_lo[3], mn_hi[3], mx_lo[3], mx_hi[3];
  int32_t nchild;
  int32_t offset;
  int32_t pad[2];
};
static_assert(sizeof(INodeSlab) == 64, "INodeSlab must be 64 bytes");

struct alignas(64) ISafe {  // box centre 0.5*(mx+mn) and half size 0.5*(mx-mn) (AABB::Safety)
  float c_lo[3], c_hi[3], hs_lo[3], hs_hi[3];
  int32_t pad[4];
};
static_assert(sizeof(ISafe) == 64, "ISafe must be 64 bytes");

struct alignas(64) IPrimSlab {  // leaf primitive box in BVH leaf order
  float mn_lo[3], mn_hi[3], mx_lo[3], mx_hi[3];
  int32_t pv;
  int32_t prim;
  int32_t shape;  // the placed volume's ShapeType (groups the FP64 shape evaluations by type)
  int32_t pad;
};
static_assert(sizeof(IPrimSlab) == 64, "IPrimSlab must be 64 bytes");

struct alignas(128) IXForm {  // placement transform as intervals + box half-lengths (shape box only)
  float t_lo[3], t_hi[3];
  float r_lo[9], r_hi[9];
  float h_lo[3], h_hi[3];  // box half-lengths; zero for other shapes
  int32_t shape;
  int32_t isin;  // first (lo, hi) pair of the shape's GeomView::isin row; -1: no interval SafetyToIn
};
static_assert(sizeof(IXForm) == 128, "IXForm must be 128 bytes");

// Rows of GeomView::isin: FP32 (lo, hi) enclosures of the doubles that each shape's
// SafetyToIn reads or derives from its parameters (derived values computed on the
// host with the device's FP64 operations), so that the interval SafetyToIn of the
// mixed kernels runs without FP64 instructions.  Flags are stored as 0/1 pairs.
namespace irow {
enum { TubeZ = 0, TubeRmax, TubeRmin, TubeHasRmin, kTubeRow };
enum { ConeDz = 0, ConeMinusConeTol, ConeTol, ConeHasRmin, ConeOuterConst, ConeOuterR, ConeOuterSlope,
       ConeOuterOffset, ConeTwoOuterTol, ConeInnerConst, ConeInnerR, ConeInnerSlope, ConeInnerOffset,
       ConeTwoInnerTol, ConeTanRMax, ConeAvgRmax, ConeInvSecRMax, ConeTanRMin, ConeAvgRmin, ConeInvSecRMin, kConeRow };
enum { TrdDz = 0, TrdHalfX, TrdFx, TrdCalfX, TrdVaryingY, TrdHalfY, TrdFy, TrdCalfY, TrdDy1, kTrdRow };
enum { TrapDz = 0, TrapA = 1, TrapB = 5, TrapC = 9, TrapD = 13, kTrapRow = 17 };
enum { SphHasRmin = 0, SphRmin, SphRmax, SphMsqMax, SphPsqMax, SphPsqMin, SphMsqMin, kSphereRow };
enum { OrbR = 0, OrbRMinusTol, OrbRPlusTol, kOrbRow };
// Polycone (full phi): number of sections n, kTolerance, the n + 1 z planes, the n section
// shifts, then one Cone row per section
enum { PconN = 0, PconTol, PconZs };
VGN_HD inline int pcon_ishift(int n) { return PconZs + n + 1; }
VGN_HD inline int pcon_icone(int n, int k) { return PconZs + 2 * n + 1 + k * kConeRow; }
}  // namespace irow

// Row layouts (doubles) of GeomView::shape per shape type.
namespace row {
// Box: BoxStruct::fDimensions
constexpr int kBoxSize = 4;
// Orb: OrbStruct::fR
constexpr int kOrbSize = 1;
// Tube: TubeStruct cached members, then its phi wedge as a Wedge block (the along vectors
// are both TubeStruct::fAlongPhi* and the wedge's; the block's last entry is fDphi)
enum { TubeRmin = 0, TubeRmax, TubeZ, TubeRmin2, TubeRmax2, TubeTolIrmin2, TubeTolOrmin2, TubeTolIrmax2,
       TubeTolOrmax2, TubeMaxVal, TubeSphi, TubeTolOz, TubeWedge, TubeDphi = TubeWedge + 8, kTubeSize };
// Boolean: BooleanStruct (BooleanStruct.h:23-25) with its placed operands resolved: the
// operation (0 union, 1 intersection, 2 subtraction), each operand's shape type and the offset
// of its shape row relative to this row, then each operand placement's transformation
// (tx, ty, tz, r0..r8), left then right
enum { BoolOp = 0, BoolLeftType, BoolLeftRow, BoolRightType, BoolRightRow, BoolLeftXf, BoolRightXf = BoolLeftXf + 12,
       kBoolSize = BoolRightXf + 12 };
// CutTube: CutTubeStruct (CutTubeStruct.h:21-46): its tube's row (infinite half-length), then
// fDz, the bottom and top cut planes (unit normal, distance), cos/sin of phi and phi+dphi, fMaxVal
enum { CutTubeDz = kTubeSize, CutTubeN0, CutTubeD0 = CutTubeN0 + 3, CutTubeN1, CutTubeD1 = CutTubeN1 + 3,
       CutTubeCos1, CutTubeSin1, CutTubeCos2, CutTubeSin2, CutTubeMaxVal, kCutTubeSize };
// Wedge block (evolution::Wedge): along vectors, normal vectors, fDPhi
enum { WedgeA1x = 0, WedgeA1y, WedgeA2x, WedgeA2y, WedgeN1x, WedgeN1y, WedgeN2x, WedgeN2y, WedgeDPhi, kWedgeSize };
// Polyhedron: PolyhedronStruct (PolyhedronStruct.h:52-80): the header (with fPhiStart and
// fPhiDelta), the bounding tube
// (a Tube row), the phi wedge fPhiWedge (a Wedge block), the arrays fZPlanes, fRMin, fRMax,
// fSameZ (nz each), fPhiSections (sides + 1 vectors), then per z segment the face counts
// (outer, phi, inner) and the offset of its first face from the row's start, and the faces
// (Quadrilaterals: plane, four side planes, four corners), outer then phi then inner
enum { PhdSides = 0, PhdNz, PhdHasPhi, PhdLargePhi, PhdTubeOffset, PhdPhiStart, PhdPhiDelta, PhdTube,
       PhdWedge = PhdTube + kTubeSize,
       PhdArrays = PhdWedge + kWedgeSize };
enum { QuadN = 0, QuadD = 3, QuadSide = 4, QuadCorner = 20, kQuadSize = 32 };  // side j: 4 doubles at QuadSide + 4 j
VGN_HD inline int phd_z(int) { return PhdArrays; }
VGN_HD inline int phd_rmin(int nz) { return PhdArrays + nz; }
VGN_HD inline int phd_rmax(int nz) { return PhdArrays + 2 * nz; }
VGN_HD inline int phd_samez(int nz) { return PhdArrays + 3 * nz; }
VGN_HD inline int phd_phisec(int nz) { return PhdArrays + 4 * nz; }
VGN_HD inline int phd_segs(int nz, int sides) { return phd_phisec(nz) + 3 * (sides + 1); }  // 4 per segment
// Torus2: TorusStruct2 (TorusStruct2.h:22-32): parameters and squares, the phi wedge, the
// bounding tube (a Tube row)
enum { TorRmin = 0, TorRmax, TorRtor, TorSphi, TorDphi, TorRmin2, TorRmax2, TorRtor2, TorWedge,
       TorTube = TorWedge + kWedgeSize, kTorusSize = TorTube + kTubeSize };
// Cone (full phi): ConeStruct cached members
enum { ConeRmin1 = 0, ConeRmax1, ConeRmin2, ConeRmax2, ConeDz, ConeOrigRmax1, ConeOrigRmax2, ConeInnerSlope,
       ConeOuterSlope, ConeInnerOffset, ConeOuterOffset, ConeInnerTol, ConeOuterTol, ConeSqRmin1, ConeSqRmin2,
       ConeSqRmax1, ConeSqRmax2, ConeTolIz, ConeInnerApex, ConeTanInnerApex, ConeOuterApex, ConeTanOuterApex,
       ConeSecRMin, ConeSecRMax, ConeInvSecRMin, ConeInvSecRMax, ConeTanRMin, ConeTanRMax, ConeZNormInner,
       ConeZNormOuter, ConeArgRmax1, ConeArgRmax2, ConeArgRmin1, ConeArgRmin2,
       // checked fSPhi, fDPhi and fAlongPhi1/2 (ConeStruct::SetAndCheck*PhiAngle), then fPhiWedge
       ConeSPhi, ConeDPhi, ConeAP1x, ConeAP1y, ConeAP2x, ConeAP2y, ConeWedge, kConeSize = ConeWedge + 9 };
// Trd (UniversalTrd): TrdStruct members and cached values; padded to 16 doubles
enum { TrdDx1 = 0, TrdDx2, TrdDy1, TrdDy2, TrdDz, TrdX2minusX1, TrdY2minusY1, TrdHalfX1plusX2, TrdHalfY1plusY2,
       TrdCalfX, TrdCalfY, TrdTolX, TrdTolY, TrdFx, TrdFy, TrdPad, kTrdSize };
// Trapezoid: half-length in z and the four side planes (PlaneShell<4>: A, B, C, D
// each of 4), then the TrapezoidStruct parameters and cached values
enum { TrapDz = 0, TrapA = 1, TrapB = 5, TrapC = 9, TrapD = 13, TrapTheta = 17, TrapPhi, TrapDy1, TrapDx1, TrapDx2,
       TrapTanAlpha1, TrapDy2, TrapDx3, TrapDx4, TrapTanAlpha2, TrapTthetaCphi, TrapTthetaSphi, kTrapSize = 32 };
// Sphere: radii, the phi wedge's along/normal vectors and raw delta-phi (a Wedge block),
// the theta cone's raw start/end angles and tangents, the fFullSphere flag; then the
// theta cone's squared tangents, bisector tangent and face slopes, the checked fDPhi,
// fDTheta and eTheta, the fFullPhiSphere / fFullThetaSphere flags (1 or 0) and the
// checked fSPhi
enum { SphRmin = 0, SphRmax, SphA1x, SphA1y, SphA2x, SphA2y, SphN1x, SphN1y, SphN2x, SphN2y, SphWedgeDPhi,
       SphSTheta, SphETheta, SphTanSTheta, SphTanETheta, SphFull, SphTanSTheta2, SphTanETheta2, SphTanBisector,
       SphSlope1, SphSlope2, SphDPhi, SphDTheta, SphEThetaChk, SphFullPhi, SphFullTheta, SphSPhi, SphPad,
       kSphereSize };
// Polycone, variable length: [0] section count n, [1, n+1] the n+1 z planes, [n+2, 2n+1]
// the section z shifts, then n cone rows of kConeSize doubles, then the raw phi start and
// total angle
constexpr int PconNSec = 0;
constexpr int PconZs   = 1;
VGN_HD inline int pcon_shift(int n) { return 2 + n; }
VGN_HD inline int pcon_cone(int n, int k) { return 2 + 2 * n + k * kConeSize; }
VGN_HD inline int pcon_phi(int n) { return pcon_cone(n, n); }  // the raw (phiStart, phiTotal)
}  // namespace row

// Plain-pointer view of the device tables, passed to kernels by value.
struct GeomView {
  const uint32_t *navind;
  const uint32_t *node_start;  // bitset: navigation indices that start a state record
  const PVRec *pv;
  const LVRec *lv;
  const int32_t *daughters;
  const NodeRec *nodes;
  const PrimRec *prims;
  const FNodeRec *fnodes;
  const FPrimRec *fprims;
  const INodeSlab *inodes;   // interval images (mixed precision), indexed like nodes
  const ISafe *inode_safe;
  const IPrimSlab *iprims;   // indexed like prims
  const ISafe *iprim_safe;
  const IXForm *ixf;         // per placed volume
  const float *isin;         // interval SafetyToIn rows (irow), (lo, hi) pairs
  const double *shape;
  const double *lv_bbox;     // per logical volume: its shape's Extent, min then max corner (6 doubles)
  uint32_t navind_words;
  int32_t n_pv;
  int32_t n_lv;
  int32_t world_pv;
  int32_t max_depth;
  uint32_t *status;  // device error word (DevError bits)
  // bounds of the device loops: traversal stack entries (<= kStackSize) and relocation
  // levels (<= kMaxLevels); lowered only to exercise the error paths (vgn_set_device_limits)
  int32_t stack_limit;
  int32_t level_limit;
};

}  // namespace vgn
