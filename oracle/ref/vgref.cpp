// vgref.cpp -- C entry points over the reference's own navigation code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/ref/Makefile compiles this file together with
// the reference's unmodified sources (VecGeom 1.2.0: BVH, ABBoxManager, GeoManager,
// NavIndexTable, LogicalVolume, the placed and unplaced shape sources, ...) against a
// scalar VecCore stand-in (oracle/ref/shim) into oracle/_ref/libvgref.so.  The tests
// use it to pin the C restatement in oracle/ and, through fixtures generated from it,
// the CUDA kernels; it is never linked into or called by the product library.
//
// The geometry comes in the flat description the product and the C oracle take
// (shape rows, placements in id order) and is built with the reference's own API:
// GeoManager::MakeInstance for the shapes, LogicalVolume::PlaceDaughter for the
// placements (source/LogicalVolume.cpp:142-148), GeoManager::SetWorldAndClose
// (source/GeoManager.cpp:192-241, which also builds the ABBoxes and the navigation
// index table), then BVHManager::Init and BVHNavigator / BVHSafetyEstimator /
// BVHLevelLocator on every logical volume with daughters, as
// test/globalbenchmarks/XRayBenchmarkFromROOTFile.cpp:203-238 sets them up.  The
// reference keeps its geometry in singletons, so one geometry exists at a time.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "VecGeom/base/SOA3D.h"
#include "VecGeom/base/Transformation3D.h"
#include "VecGeom/management/BVHManager.h"
#include "VecGeom/management/GeoManager.h"
#include "VecGeom/management/NavIndexTable.h"
#include "VecGeom/navigation/BVHLevelLocator.h"
#include "VecGeom/navigation/BVHNavigator.h"
#include "VecGeom/navigation/BVHSafetyEstimator.h"
#include "VecGeom/navigation/GlobalLocator.h"
#include "VecGeom/navigation/NavStatePool.h"
#include "VecGeom/navigation/NavigationState.h"
#include "VecGeom/volumes/LogicalVolume.h"
#include "VecGeom/volumes/PlacedVolume.h"
#include "VecGeom/volumes/BooleanVolume.h"
#include "VecGeom/volumes/UnplacedBox.h"
#include "VecGeom/volumes/UnplacedCone.h"
#include "VecGeom/volumes/UnplacedCutTube.h"
#include "VecGeom/volumes/UnplacedOrb.h"
#include "VecGeom/volumes/UnplacedPolycone.h"
#include "VecGeom/volumes/UnplacedPolyhedron.h"
#include "VecGeom/volumes/UnplacedTorus2.h"
#include "VecGeom/volumes/UnplacedSphere.h"
#include "VecGeom/volumes/UnplacedTrapezoid.h"
#include "VecGeom/volumes/UnplacedTrd.h"
#include "VecGeom/volumes/UnplacedTube.h"

using namespace vecgeom;

static_assert(sizeof(NavStateIndex) == 12, "NavStateIndex is the 12-byte index state");

extern "C" {

typedef struct {
  uint32_t nav_ind;
  uint32_t last_exited;
  uint8_t on_boundary;
  uint8_t pad[3];
} vgref_state;

// BVH arrays of one logical volume (vgref_bvh.cpp, which reads the BVH's members)
int vgref_bvh_read(const void *bvh, int *depth, int *n_nodes, int *n_prims, int *prim_id, int *offset, int *nchild,
                   double *nodes_minmax, double *prims_minmax);
}

namespace {

std::vector<LogicalVolume *> g_lv;  // logical volumes of the current geometry, by id
bool g_ready = false;

void set_err(char *err, int errlen, const char *msg)
{
  if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", msg);
}

// the reference's shape for one row of the flat description (numbering of vgn_shape_type)
VUnplacedVolume *make_shape(int type, const double *p)
{
  switch (type) {
  case 0:
    return GeoManager::MakeInstance<UnplacedBox>(p[0], p[1], p[2]);
  case 1:
    return GeoManager::MakeInstance<UnplacedTube>(p[0], p[1], p[2], p[3], p[4]);
  case 2:
    return GeoManager::MakeInstance<UnplacedCone>(p[0], p[1], p[2], p[3], p[4], p[5], p[6]);
  case 3:
    return GeoManager::MakeInstance<UnplacedTrd>(p[0], p[1], p[2], p[3], p[4]);
  case 4:
    return GeoManager::MakeInstance<UnplacedTrapezoid>(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9],
                                                       p[10]);
  case 5:
    return GeoManager::MakeInstance<UnplacedSphere>(p[0], p[1], p[2], p[3], p[4], p[5]);
  case 6: {
    const int nz = (int)p[2];
    return GeoManager::MakeInstance<UnplacedPolycone>(p[0], p[1], nz, p + 3, p + 3 + nz, p + 3 + 2 * nz);
  }
  case 7:
    return GeoManager::MakeInstance<UnplacedOrb>(p[0]);
  case 8:
    return GeoManager::MakeInstance<UnplacedCutTube>(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9],
                                                     p[10]);
  case 11:
    return GeoManager::MakeInstance<UnplacedTorus2>(p[0], p[1], p[2], p[3], p[4]);
  case 10: {
    const int nz = (int)p[3];
    return GeoManager::MakeInstance<UnplacedPolyhedron>(p[0], p[1], (int)p[2], nz, p + 4, p + 4 + nz, p + 4 + 2 * nz);
  }
  default:
    return nullptr;
  }
}

inline NavStateIndex to_ref(const vgref_state &s)
{
  NavStateIndex r;
  std::memcpy(&r, &s, sizeof(r));
  return r;
}

inline vgref_state from_ref(const NavStateIndex &s)
{
  vgref_state r;
  std::memcpy(&r, &s, sizeof(r));
  r.pad[0] = r.pad[1] = r.pad[2] = 0;
  r.on_boundary &= 1;
  return r;
}

template <typename F>
void parallel_for(long n, int nthreads, F &&f)
{
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 1024) nt = 1;
  if (nt == 1) {
    f(0L, n);
    return;
  }
  std::vector<std::thread> th;
  const long chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const long lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([&f, lo, hi] { f(lo, hi); });
  }
  for (auto &x : th) x.join();
}

inline VNavigator const *navigator_of(NavStateIndex const &s)
{
  return s.Top()->GetLogicalVolume()->GetNavigator();
}

} // namespace

extern "C" {

// cache_depth: GeoManager::SetTransformationCacheDepth before closing (0 = every level cached)
int vgref_geom_create(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params, int n_params,
                      int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans, int world_pv,
                      int cache_depth, char *err, int errlen)
{
  if (n_lv <= 0 || n_pv <= 0 || world_pv < 0 || world_pv >= n_pv || pv_mother[world_pv] != -1) {
    set_err(err, errlen, "empty geometry or bad world placement");
    return 1;
  }
  GeoManager::Instance().Clear();
  g_lv.assign((size_t)n_lv, nullptr);
  g_ready = false;
  for (int i = 0; i < n_lv; ++i) {
    if (lv_param_off[i] < 0 || lv_param_off[i] >= n_params) {
      set_err(err, errlen, "shape parameters out of range");
      return 1;
    }
    VUnplacedVolume *u = nullptr;
    if (lv_shape[i] == 9) {  // boolean: place its operands now, as a boolean's creator does
      const double *p = params + lv_param_off[i];
      VPlacedVolume const *operand[2] = {nullptr, nullptr};
      for (int k = 0; k < 2; ++k) {
        const int pv = (int)p[1 + k];
        if (pv < 0 || pv >= n_pv || pv_mother[pv] != -2 || pv_lv[pv] < 0 || pv_lv[pv] >= i) {
          set_err(err, errlen, "bad boolean operand");
          return 1;
        }
        const double *t = pv_trans + 12 * (size_t)pv;
        auto *xf = new Transformation3D(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], t[9], t[10], t[11]);
        const std::string name = "op" + std::to_string(pv);
        operand[k]             = g_lv[(size_t)pv_lv[pv]]->Place(name.c_str(), xf);
        if (operand[k]->id() != (unsigned)pv) {  // ids count up in creation order
          set_err(err, errlen, "this driver creates operands with their boolean: their ids must follow that order");
          return 1;
        }
      }
      switch ((int)p[0]) {
      case 0: u = new UnplacedBooleanVolume<kUnion>(kUnion, operand[0], operand[1]); break;
      case 1: u = new UnplacedBooleanVolume<kIntersection>(kIntersection, operand[0], operand[1]); break;
      case 2: u = new UnplacedBooleanVolume<kSubtraction>(kSubtraction, operand[0], operand[1]); break;
      default: break;
      }
    } else {
      u = make_shape(lv_shape[i], params + lv_param_off[i]);
    }
    if (!u) {
      set_err(err, errlen, "unsupported shape type");
      return 1;
    }
    const std::string name = "lv" + std::to_string(i);
    g_lv[(size_t)i]        = new LogicalVolume(name.c_str(), u);
  }
  VPlacedVolume *world = nullptr;
  // placements in id order: VPlacedVolume ids count up in creation order (source/PlacedVolume.cpp:32)
  for (int i = 0; i < n_pv; ++i) {
    if (pv_lv[i] < 0 || pv_lv[i] >= n_lv || pv_mother[i] < -2 || pv_mother[i] >= n_lv) {
      set_err(err, errlen, "placement refers to an unknown logical volume");
      return 1;
    }
    if (pv_mother[i] == -2) continue;  // a boolean operand, placed with its boolean
    const double *t = pv_trans + 12 * (size_t)i;
    auto *xf = new Transformation3D(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], t[9], t[10], t[11]);
    if (pv_mother[i] < 0) {
      if (i != world_pv) {
        set_err(err, errlen, "second placement without a mother");
        return 1;
      }
      world = g_lv[(size_t)pv_lv[i]]->Place("world", xf);
    } else {
      const std::string name = "pv" + std::to_string(i);
      g_lv[(size_t)pv_mother[i]]->PlaceDaughter(name.c_str(), g_lv[(size_t)pv_lv[i]], xf);
    }
  }
  // GeoManager::Clear keeps the previous geometry's transformation cache depth
  // (source/GeoManager.cpp:355-378); a fresh process starts at 0 (cache every level)
  GeoManager::Instance().SetTransformationCacheDepth(cache_depth);
  GeoManager::Instance().SetWorldAndClose(world);
  BVHManager::Init();
  for (auto &item : GeoManager::Instance().GetLogicalVolumesMap()) {
    LogicalVolume *lv = item.second;
    if (lv->GetDaughters().size() > 0) {
      lv->SetNavigator(BVHNavigator<>::Instance());
      lv->SetSafetyEstimator(BVHSafetyEstimator::Instance());
      lv->SetLevelLocator(BVHLevelLocator::GetInstance());
    }
  }
  g_ready = true;
  return 0;
}

const uint32_t *vgref_navindex(size_t *n_words)
{
  if (!g_ready) return nullptr;
  *n_words = NavIndexTable::Instance()->GetTableSize() / sizeof(NavIndex_t);
  return NavIndexTable::Instance()->GetTable();
}

int vgref_max_depth(void)
{
  return g_ready ? GeoManager::Instance().getMaxDepth() : -1;
}

int vgref_bvh_info(int lv, int *depth, int *n_nodes, int *n_prims)
{
  if (!g_ready || lv < 0 || lv >= (int)g_lv.size()) return 1;
  BVH const *b = BVHManager::GetBVH(lv);
  if (!b) return 1;
  return vgref_bvh_read(b, depth, n_nodes, n_prims, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int vgref_bvh_arrays(int lv, int *prim_id, int *offset, int *nchild, double *nodes_minmax, double *prims_minmax)
{
  if (!g_ready || lv < 0 || lv >= (int)g_lv.size()) return 1;
  BVH const *b = BVHManager::GetBVH(lv);
  if (!b) return 1;
  int d, nn, np;
  return vgref_bvh_read(b, &d, &nn, &np, prim_id, offset, nchild, nodes_minmax, prims_minmax);
}

// VUnplacedVolume queries (op numbering of vgn_shape_op); stepmax NULL = kInfLength
int vgref_shape_batch(int lv, int op, long n, const double *px, const double *py, const double *pz, const double *dx,
                      const double *dy, const double *dz, const double *stepmax, double *out)
{
  if (!g_ready || lv < 0 || lv >= (int)g_lv.size() || op < 0 || op > 5) return 1;
  VUnplacedVolume const *u = g_lv[(size_t)lv]->GetUnplacedVolume();
  for (long i = 0; i < n; ++i) {
    const Vector3D<Precision> p(px[i], py[i], pz[i]);
    const double sm = stepmax ? stepmax[i] : kInfLength;
    switch (op) {
    case 0:
      out[i] = u->DistanceToIn(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), sm);
      break;
    case 1:
      out[i] = u->DistanceToOut(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), sm);
      break;
    case 2:
      out[i] = u->SafetyToIn(p);
      break;
    case 3:
      out[i] = u->SafetyToOut(p);
      break;
    case 4:
      out[i] = u->Contains(p) ? 1.0 : 0.0;
      break;
    default:
      out[i] = (double)u->Inside(p);
      break;
    }
  }
  return 0;
}

// Per-track scalar interface: ComputeStepAndSafetyAndPropagatedState (VNavigator.h:1014-1064),
// or ComputeStepAndPropagatedState (VNavigator.h:436-492) when calcsafety is 0, or ComputeStep
// (VNavigator.h:494-540) when relocate is 0; the navigator is the one of the track's volume.
// Returns the seconds spent in the navigator calls.
double vgref_step_batch(long n, const double *px, const double *py, const double *pz, const double *dx,
                        const double *dy, const double *dz, const double *slimit, const vgref_state *in,
                        vgref_state *out, double *step, double *safety, int calcsafety, int relocate, int nthreads)
{
  if (!g_ready) return -1.0;
  const auto t0 = std::chrono::steady_clock::now();
  parallel_for(n, nthreads, [&](long lo, long hi) {
    for (long i = lo; i < hi; ++i) {
      const NavStateIndex s = to_ref(in[i]);
      NavStateIndex o;
      const Vector3D<Precision> p(px[i], py[i], pz[i]), d(dx[i], dy[i], dz[i]);
      VNavigator const *nav = navigator_of(s);
      if (!relocate) {
        step[i] = nav->ComputeStep(p, d, slimit[i], s, o);
      } else if (calcsafety) {
        Precision sf = 0.;
        step[i]      = nav->ComputeStepAndSafetyAndPropagatedState(p, d, slimit[i], s, o, true, sf);
        safety[i]    = sf;
      } else {
        step[i] = nav->ComputeStepAndPropagatedState(p, d, slimit[i], s, o);
      }
      out[i] = from_ref(o);
    }
  });
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Vector interface: ComputeStepsAndSafetiesAndPropagatedStates over SOA3D and NavStatePool
// (VNavigator.h:913-941), called on the navigator of the first track's volume, as its
// callers do (test/benchmark/NavigationKernelBenchmarker.cpp:360-368).  Every track of
// a chunk must sit in that volume.  Each thread takes one contiguous chunk of the batch.
// Returns the seconds spent in the navigator calls (pool set-up excluded).
double vgref_step_vector(long n, const double *px, const double *py, const double *pz, const double *dx,
                         const double *dy, const double *dz, const double *slimit, const vgref_state *in,
                         vgref_state *out, double *step, const uint8_t *calcsafeties, double *safety, int nthreads)
{
  if (!g_ready || n <= 0) return -1.0;
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 1024) nt = 1;
  const long chunk = (n + nt - 1) / nt;
  const int depth  = GeoManager::Instance().getMaxDepth();
  struct Piece {
    long lo, hi;
    NavStatePool *inp, *outp;
    std::vector<bool> calc;
    bool *calcp;
  };
  std::vector<Piece> pieces;
  for (int t = 0; t < nt; ++t) {
    const long lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    Piece pc{lo, hi, new NavStatePool((int)(hi - lo), depth), new NavStatePool((int)(hi - lo), depth), {}, nullptr};
    for (long i = lo; i < hi; ++i) *(*pc.inp)[(int)(i - lo)] = to_ref(in[i]);
    pc.calcp = new bool[(size_t)(hi - lo)];
    for (long i = lo; i < hi; ++i) pc.calcp[i - lo] = calcsafeties ? calcsafeties[i] != 0 : false;
    pieces.push_back(std::move(pc));
  }
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (auto &pc : pieces) {
    th.emplace_back([&pc, px, py, pz, dx, dy, dz, slimit, step, safety] {
      const long m = pc.hi - pc.lo;
      SOA3D<Precision> pts(const_cast<double *>(px + pc.lo), const_cast<double *>(py + pc.lo),
                           const_cast<double *>(pz + pc.lo), (size_t)m);
      SOA3D<Precision> dirs(const_cast<double *>(dx + pc.lo), const_cast<double *>(dy + pc.lo),
                            const_cast<double *>(dz + pc.lo), (size_t)m);
      VNavigator const *nav = navigator_of(*(*pc.inp)[0]);
      nav->ComputeStepsAndSafetiesAndPropagatedStates(pts, dirs, slimit + pc.lo, *pc.inp, *pc.outp, step + pc.lo,
                                                      pc.calcp, safety + pc.lo);
    });
  }
  for (auto &x : th) x.join();
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (auto &pc : pieces) {
    for (long i = pc.lo; i < pc.hi; ++i) out[i] = from_ref(*(*pc.outp)[(int)(i - pc.lo)]);
    delete pc.inp;
    delete pc.outp;
    delete[] pc.calcp;
  }
  return secs;
}

// VSafetyEstimatorHelper::ComputeSafety (VSafetyEstimator.h:98-107) with the estimator of
// the track's volume
void vgref_safety_batch(long n, const double *px, const double *py, const double *pz, const vgref_state *in,
                        double *safety, int nthreads)
{
  if (!g_ready) return;
  parallel_for(n, nthreads, [&](long lo, long hi) {
    for (long i = lo; i < hi; ++i) {
      const NavStateIndex s = to_ref(in[i]);
      safety[i] = s.Top()->GetLogicalVolume()->GetSafetyEstimator()->ComputeSafety(Vector3D<Precision>(px[i], py[i],
                                                                                                      pz[i]),
                                                                                  s);
    }
  });
}

// GlobalLocator::LocateGlobalPoint from the world, top = true (GlobalLocator.h:35-82)
void vgref_locate_batch(long n, const double *px, const double *py, const double *pz, vgref_state *out, int nthreads)
{
  if (!g_ready) return;
  VPlacedVolume const *world = GeoManager::Instance().GetWorld();
  parallel_for(n, nthreads, [&](long lo, long hi) {
    for (long i = lo; i < hi; ++i) {
      NavStateIndex s;
      GlobalLocator::LocateGlobalPoint(world, Vector3D<Precision>(px[i], py[i], pz[i]), s, true);
      out[i] = from_ref(s);
    }
  });
}

// BVH::ApproachNextDaughter (BVH.cpp:395-449) of logical volume lv[i]'s BVH for each track:
// local point and direction in that volume, step in/out, last[i] the id of the last exited
// placed volume or -1.  Returns 1 if a volume has no BVH.
int vgref_approach_batch(long n, const int *lv, const double *px, const double *py, const double *pz,
                         const double *dx, const double *dy, const double *dz, const int *last, double *step,
                         int nthreads)
{
  if (!g_ready) return 1;
  for (long i = 0; i < n; ++i)
    if (lv[i] < 0 || lv[i] >= (int)g_lv.size() || !BVHManager::GetBVH(lv[i])) return 1;
  parallel_for(n, nthreads, [&](long lo, long hi) {
    for (long i = lo; i < hi; ++i) {
      VPlacedVolume const *lastpv = last[i] >= 0 ? GeoManager::Instance().FindPlacedVolume(last[i]) : nullptr;
      BVHManager::GetBVH(lv[i])->ApproachNextDaughter(Vector3D<Precision>(px[i], py[i], pz[i]),
                                                      Vector3D<Precision>(dx[i], dy[i], dz[i]), step[i], lastpv);
    }
  });
  return 0;
}

// VUnplacedVolume::Extent of logical volume lv's shape: min then max corner
int vgref_extent(int lv, double *out6)
{
  if (!g_ready || lv < 0 || lv >= (int)g_lv.size()) return 1;
  Vector3D<Precision> mn, mx;
  g_lv[(size_t)lv]->GetUnplacedVolume()->Extent(mn, mx);
  for (int k = 0; k < 3; ++k) out6[k] = mn[k], out6[3 + k] = mx[k];
  return 0;
}

int vgref_ncores(void)
{
  return (int)std::max(1u, std::thread::hardware_concurrency());
}

} // extern "C"
