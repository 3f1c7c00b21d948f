// host_geometry.cpp -- closes a geometry on the host and lays out the
// device tables (geom_types.h).
//
// The BVH construction has to produce the same tree as the reference's
// (source/BVH.cpp:48-87, 242-385): leaf candidate order decides which of two
// equidistant daughters a step reports, so the split rule (SAH with the
// reference's balance term), the std::sort ordering key and std::partition
// are kept.  The navigation index table must be laid out exactly as the
// reference's (source/NavIndexTable.cpp:9-99) because NavStateIndex values
// are offsets into it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

#include "../../include/vgnav.h"
#include "host_geometry.h"

namespace vgn {

static constexpr double kTol = 1e-9;

void xform_identity(HostXForm &m)
{
  std::memset(&m, 0, sizeof(m));
  m.r[0] = m.r[4] = m.r[8] = 1.;
  m.identity           = true;
  m.has_rot = m.has_trans = false;
}

// Transformation3D(tx,ty,tz,r0..r8) + SetProperties (source/Transformation3D.cpp:52-61, 117-126, 170-182)
HostXForm xform_from12(const double *a)
{
  HostXForm m;
  for (int i = 0; i < 3; ++i) m.t[i] = a[i];
  for (int i = 0; i < 9; ++i) m.r[i] = a[3 + i];
  m.has_trans = std::fabs(m.t[0]) > kTol || std::fabs(m.t[1]) > kTol || std::fabs(m.t[2]) > kTol;
  int code    = 0;
  for (int i = 0; i < 9; ++i) code |= (1 << i) * (std::fabs(m.r[i]) > kTol);
  if (code == 0x111 && m.r[0] == 1. && m.r[4] == 1. && m.r[8] == 1.) code = 0x200;
  m.has_rot  = code != 0x200;
  m.identity = !m.has_trans && !m.has_rot;
  return m;
}

// Transformation3D::MultiplyFromRight (Transformation3D.h:878-946)
void xform_multiply_from_right(HostXForm &m, const HostXForm &rhs)
{
  if (rhs.identity) return;
  m.identity = false;
  if (rhs.has_trans) {
    m.has_trans = true;
    for (int row = 0; row < 3; ++row) {
      m.t[row] += m.r[3 * row + 0] * rhs.t[0];
      m.t[row] += m.r[3 * row + 1] * rhs.t[1];
      m.t[row] += m.r[3 * row + 2] * rhs.t[2];
    }
  }
  if (rhs.has_rot) {
    m.has_rot = true;
    for (int row = 0; row < 3; ++row) {
      double *r      = m.r + 3 * row;
      const double x = r[0], y = r[1], z = r[2];
      r[0] = x * rhs.r[0];
      r[1] = x * rhs.r[1];
      r[2] = x * rhs.r[2];
      r[0] += y * rhs.r[3];
      r[1] += y * rhs.r[4];
      r[2] += y * rhs.r[5];
      r[0] += z * rhs.r[6];
      r[1] += z * rhs.r[7];
      r[2] += z * rhs.r[8];
    }
  }
}

// InverseTransform (Transformation3D.h:793-827)
Vec3 xform_inverse_transform(const HostXForm &m, const Vec3 &l)
{
  double o[3];
  for (int row = 0; row < 3; ++row) {
    double v = m.t[row];
    v += l.x * m.r[3 * row + 0];
    v += l.y * m.r[3 * row + 1];
    v += l.z * m.r[3 * row + 2];
    o[row] = v;
  }
  return {o[0], o[1], o[2]};
}

namespace {

inline double vmin(double a, double b) { return a < b ? a : b; }  // vecCore Min
inline double vmax(double a, double b) { return a > b ? a : b; }  // vecCore Max
inline double comp(const Vec3 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

Box3 box_union(const Box3 &a, const Box3 &b)
{
  return {{vmin(a.mn.x, b.mn.x), vmin(a.mn.y, b.mn.y), vmin(a.mn.z, b.mn.z)},
          {vmax(a.mx.x, b.mx.x), vmax(a.mx.y, b.mx.y), vmax(a.mx.z, b.mx.z)}};
}

double box_area(const Box3 &b)
{
  const double e0 = b.mx.x - b.mn.x, e1 = b.mx.y - b.mn.y, e2 = b.mx.z - b.mn.z;
  return 2. * (e0 * e1 + e1 * e2 + e2 * e0);
}

// SAH sort key: centroid + 0.01 * (centroid - min) (BVH.cpp:284-291)
Vec3 sah_key(const Box3 &b)
{
  const Vec3 c{0.5 * (b.mx.x + b.mn.x), 0.5 * (b.mx.y + b.mn.y), 0.5 * (b.mx.z + b.mn.z)};
  return {c.x + 0.01 * (c.x - b.mn.x), c.y + 0.01 * (c.y - b.mn.y), c.z + 0.01 * (c.z - b.mn.z)};
}

bool less3d(const Vec3 &l, const Vec3 &r, int ax)
{
  const int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  return comp(l, ax) < comp(r, ax) ||
         (comp(l, ax) == comp(r, ax) &&
          (comp(l, a1) < comp(r, a1) || (comp(l, a1) == comp(r, a1) && comp(l, a2) < comp(r, a2))));
}

class BVHBuilder {
public:
  BVHBuilder(const std::vector<Box3> &boxes, HostBVH &bvh) : boxes_(boxes), bvh_(bvh)
  {
    keys_.resize(boxes.size());
    for (size_t i = 0; i < boxes.size(); ++i) keys_[i] = sah_key(boxes[i]);
  }

  void build()
  {
    const int n = (int)boxes_.size();
    bvh_.prim_id.resize(n);
    std::iota(bvh_.prim_id.begin(), bvh_.prim_id.end(), 0);
    const int half = n / 2;
    int depth      = half > 0 ? (int)std::log2((double)half) : 0;
    bvh_.depth     = std::min(std::max(depth, 0), 32);
    const unsigned nodes = (2u << bvh_.depth) - 1;
    bvh_.nchild.assign(nodes, 0);
    bvh_.offset.assign(nodes, -1);
    bvh_.nodes.assign(nodes, Box3{{0, 0, 0}, {0, 0, 0}});
    int *base = bvh_.prim_id.data();
    compute_nodes(0, base, base + n, nodes);
    for (unsigned id = 0; id < nodes / 2; ++id)
      if (bvh_.nchild[id] > 8 && bvh_.nchild[id] == bvh_.nchild[2 * id + 1] + bvh_.nchild[2 * id + 2])
        bvh_.nchild[id] = -1;
  }

private:
  const std::vector<Box3> &boxes_;
  std::vector<Vec3> keys_;
  HostBVH &bvh_;

  void compute_nodes(unsigned id, int *first, int *last, unsigned nodes)
  {
    if (id >= nodes) return;
    bvh_.nchild[id] = (int)(last - first);
    bvh_.offset[id] = (int)(first - bvh_.prim_id.data());
    if (first == last) return;
    Box3 b = boxes_[*first];
    for (int *it = first + 1; it != last; ++it) b = box_union(b, boxes_[*it]);
    bvh_.nodes[id] = b;
    if (first + 1 == last) return;
    int *pivot = sah_split(first, last);
    compute_nodes(2 * id + 1, first, pivot, nodes);
    compute_nodes(2 * id + 2, pivot, last, nodes);
  }

  // surfaceAreaHeuristic (BVH.cpp:275-329)
  int *sah_split(int *begin, int *end)
  {
    const long nObj   = end - begin;
    int bestAxis      = -1;
    int bestObject    = -1;
    double bestMetric = (double)nObj;
    std::vector<double> left(nObj), right(nObj);
    for (int axis = 0; axis <= 2; ++axis) {
      std::sort(begin, end, [&](int a, int b) { return less3d(keys_[a], keys_[b], axis); });
      std::fill(left.begin(), left.end(), 0.);
      Box3 box = boxes_[begin[0]];
      for (long k = 1; k < nObj; ++k) {
        left[k] = box_area(box);
        box     = box_union(box, boxes_[begin[k]]);
      }
      Box3 box2 = boxes_[begin[nObj - 1]];
      for (long k = nObj - 1; k >= 0; --k) {
        box2     = box_union(box2, boxes_[begin[k]]);
        right[k] = box_area(box2);
      }
      const double tot = right[0];
      for (long k = 0; k < nObj; ++k) {
        const double l = left[k] / tot, r = right[k] / tot;
        const long bal = nObj / 2 - k / nObj;  // integer arithmetic as in the reference
        const double metric = l * (double)k + r * (double)(nObj - k) + 0.1 * (double)(bal < 0 ? -bal : bal);
        if (metric < bestMetric) {
          bestMetric = metric;
          bestAxis   = axis;
          bestObject = begin[k];
        }
      }
    }
    if (bestAxis == -1) return end;
    const Vec3 pk = keys_[bestObject];
    return std::partition(begin, end, [&](int i) { return less3d(keys_[i], pk, bestAxis); });
  }
};

// ---- navigation index table (source/NavIndexTable.cpp:9-99) ----
class NavIndexBuilder {
public:
  explicit NavIndexBuilder(HostGeometry &g) : g_(g) {}

  void build()
  {
    counting_ = true;
    bytes_    = sizeof(uint32_t);
    current_  = 1;
    visit(g_.world_pv, 0, 0, 0);
    g_.navind.assign(bytes_ / sizeof(uint32_t) + 1, 0u);  // NavIndexTable::AllocateTable size
    g_.node_start.assign((g_.navind.size() + 31) / 32, 0u);
    counting_ = false;
    current_  = 1;
    visit(g_.world_pv, 0, 0, 0);
  }

private:
  HostGeometry &g_;
  bool counting_ = true;
  size_t bytes_  = 4;
  uint32_t current_ = 1;
  int32_t path_[kMaxLevels + 2] = {};

  uint32_t apply(int level, uint32_t mother, int dind)
  {
    const int pv            = path_[level];
    const HostLV &lv        = g_.lv[g_.pv[pv].lv];
    const uint16_t nd       = (uint16_t)lv.daughters.size();
    const uint32_t new_mother = current_;
    const size_t before     = counting_ ? bytes_ / 4 : current_;
    const uint32_t dindices = 3 + nd + ((nd + 1) & 1);
    const bool pad          = ((before + dindices) * 4) % 8 != 0;
    // GeoManager::CloseGeometry: the cache depth limit is the geometry's level count when
    // unset or larger (GeoManager.cpp:220-221); deeper nodes cache no matrix
    // (NavIndexTable.cpp:18).  The counting pass sizes the pad word even without a matrix.
    const int levels = g_.max_depth + 1;
    const int limit  = (g_.cache_depth == 0 || g_.cache_depth > levels) ? levels : g_.cache_depth;
    const bool cache = !(limit > 0 && level > limit);
    if (counting_) {
      bytes_ += (dindices + (pad ? 1 : 0)) * 4 + (cache ? 12 * 8 : 0);
      return 0;
    }
    uint32_t *tab      = g_.navind.data();
    g_.node_start[current_ >> 5] |= 1u << (current_ & 31);
    tab[current_]      = mother;
    if (mother > 0) tab[mother + 3 + dind] = current_;
    tab[current_ + 1]  = (uint32_t)pv;
    uint8_t *bytes     = reinterpret_cast<uint8_t *>(&tab[current_ + 2]);
    bytes[0]           = (uint8_t)level;
    bytes[1]           = 0;
    std::memcpy(bytes + 2, &nd, 2);
    for (int i = 0; i < nd; ++i) tab[current_ + 3 + i] = 0;
    current_ += dindices;
    if (!cache) return new_mother;
    // global matrix of this level: identity times placements of levels 1..level
    HostXForm mat;
    xform_identity(mat);
    for (int i = 1; i <= level; ++i) xform_multiply_from_right(mat, g_.pv[path_[i]].xf);
    bytes[1] = (uint8_t)(0x04 + 0x02 * (mat.has_trans ? 1 : 0) + (mat.has_rot ? 1 : 0));
    if (pad) current_++;
    double *m = reinterpret_cast<double *>(&tab[current_]);
    for (int i = 0; i < 3; ++i) m[i] = mat.t[i];
    for (int i = 0; i < 9; ++i) m[3 + i] = mat.r[i];
    current_ += 24;
    return new_mother;
  }

  void visit(int pv, int level, uint32_t mother, int dind)
  {
    path_[level]        = pv;
    const uint32_t nm   = apply(level, mother, dind);
    const HostLV &lv    = g_.lv[g_.pv[pv].lv];
    for (size_t i = 0; i < lv.daughters.size(); ++i) visit(lv.daughters[i], level + 1, nm, (int)i);
  }
};

int depth_below(const HostGeometry &g, int pv, int level)
{
  int d = level;
  for (int c : g.lv[g.pv[pv].lv].daughters) d = std::max(d, depth_below(g, c, level + 1));
  return d;
}

// ABBoxManager::ComputeABBox (source/ABBoxManager.cpp:109-142)
Box3 compute_abbox(const HostGeometry &g, int pv)
{
  const HostLV &lv = g.lv[g.pv[pv].lv];
  Vec3 lower, upper;
  shape_extent(lv.shape, &g.shape[lv.shape_row], lower, upper);
  const Vec3 delta{upper.x - lower.x, upper.y - lower.y, upper.z - lower.z};
  double minx = 1.7976931348623157e308, miny = minx, minz = minx;
  double maxx = -minx, maxy = -minx, maxz = -minx;
  for (int x = 0; x <= 1; ++x)
    for (int y = 0; y <= 1; ++y)
      for (int z = 0; z <= 1; ++z) {
        const Vec3 corner{lower.x + x * delta.x, lower.y + y * delta.y, lower.z + z * delta.z};
        const Vec3 tc = xform_inverse_transform(g.pv[pv].xf, corner);
        minx = std::min(minx, tc.x);
        miny = std::min(miny, tc.y);
        minz = std::min(minz, tc.z);
        maxx = std::max(maxx, tc.x);
        maxy = std::max(maxy, tc.y);
        maxz = std::max(maxz, tc.z);
      }
  return {{minx - 1E-3, miny - 1E-3, minz - 1E-3}, {maxx + 1E-3, maxy + 1E-3, maxz + 1E-3}};
}

// outward rounding of a double to float
inline float round_down(double v)
{
  float f = (float)v;
  if ((double)f > v) f = std::nextafter(f, -INFINITY);
  return f;
}
inline float round_up(double v)
{
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, INFINITY);
  return f;
}

}  // namespace

void build_interval_images(HostGeometry &g);

// Boolean solids (vgn_shape_type VGN_BOOLEAN): each operand placement (pv_mother
// VGN_BOOLEAN_OPERAND, anywhere in the placement list) is used by exactly one boolean
// (UnplacedBooleanVolume.h:59 holds its own placed operands); an operand's logical volume
// precedes its boolean, has no daughters and is a primitive or a boolean of primitives.  Fills each boolean's row with its operands' shape types, row
// offsets (relative to the boolean's row) and placement transforms.
static int link_booleans(HostGeometry &g, const vgn_geometry_desc &d, std::string &err)
{
  int used = 0, n_operands = 0;
  std::vector<char> taken(d.n_placed, 0);
  for (int i = 0; i < d.n_placed; ++i)
    if (d.pv_mother[i] == VGN_BOOLEAN_OPERAND) ++n_operands;
  for (size_t l = 0; l < g.lv.size(); ++l) {
    if (g.lv[l].shape != kBoolean) continue;
    g.booleans = true;
    double *b  = &g.shape[g.lv[l].shape_row];
    for (int k = 0; k < 2; ++k) {
      const int rowi = k == 0 ? row::BoolLeftRow : row::BoolRightRow;
      const int pv   = (int)b[rowi];
      if (pv >= d.n_placed || d.pv_mother[pv] != VGN_BOOLEAN_OPERAND || taken[pv]++) {
        err = "a boolean operand must be a placement whose mother is VGN_BOOLEAN_OPERAND, used once";
        return VGN_ERR_ARG;
      }
      ++used;
      const int olv = d.pv_logical[pv];
      if (olv >= (int)l) {
        err = "a boolean operand's logical volume must precede the boolean";
        return VGN_ERR_ARG;
      }
      const HostLV &o = g.lv[olv];
      if (!o.daughters.empty()) {
        err = "a boolean operand must have no daughters";
        return VGN_ERR_ARG;
      }
      if (o.shape == kBoolean) {
        const double *ob = &g.shape[o.shape_row];
        if (ob[row::BoolLeftType] == kBoolean || ob[row::BoolRightType] == kBoolean) {
          err = "booleans nest two levels at most";
          return VGN_ERR_UNSUPPORTED;
        }
      }
      b[k == 0 ? row::BoolLeftType : row::BoolRightType] = o.shape;
      b[rowi]                                           = (double)(o.shape_row - g.lv[l].shape_row);
      std::copy(d.pv_transform + 12 * (size_t)pv, d.pv_transform + 12 * (size_t)pv + 12,
                b + (k == 0 ? row::BoolLeftXf : row::BoolRightXf));
    }
    g.sections = g.sections || shape_row_has_sections(kBoolean, b);
  }
  if (used != n_operands) {
    err = "a boolean operand placement is not used by exactly one boolean";
    return VGN_ERR_ARG;
  }
  return VGN_OK;
}

int build_host_geometry(const vgn_geometry_desc &d, HostGeometry &g, std::string &err, int32_t cache_depth)
{
  if (cache_depth < 0) {
    err = "negative transformation cache depth";
    return VGN_ERR_ARG;
  }
  g.cache_depth = cache_depth;
  if (d.n_logical <= 0 || d.n_placed <= 0 || !d.lv_shape || !d.lv_param_offset || !d.params || !d.pv_logical ||
      !d.pv_mother || !d.pv_transform) {
    err = "geometry description has empty or null arrays";
    return VGN_ERR_ARG;
  }
  if (d.world_placed < 0 || d.world_placed >= d.n_placed || d.pv_mother[d.world_placed] != -1) {
    err = "world placement index invalid or world has a mother";
    return VGN_ERR_ARG;
  }
  g.lv.assign(d.n_logical, HostLV());
  g.pv.assign(d.n_placed, HostPV());
  g.shape.clear();
  g.world_pv = d.world_placed;
  for (int i = 0; i < d.n_logical; ++i) {
    const int off = d.lv_param_offset[i];
    if (off < 0 || off >= d.n_params) {
      err = "shape parameter offset out of range for logical volume " + std::to_string(i);
      return VGN_ERR_ARG;
    }
    const int np = shape_param_count(d.lv_shape[i], d.params + off, d.n_params - off);
    if (np < 0 || off + np > d.n_params) {
      err = "unsupported shape type or truncated parameters for logical volume " + std::to_string(i);
      return VGN_ERR_UNSUPPORTED;
    }
    g.lv[i].shape     = d.lv_shape[i];
    g.lv[i].shape_row = (int32_t)g.shape.size();
    const int rc      = shape_make_row(d.lv_shape[i], d.params + off, d.n_params - off, g.shape, err);
    if (rc) {
      err = "logical volume " + std::to_string(i) + ": " + err;
      return rc;
    }
    g.sections = g.sections || shape_row_has_sections(d.lv_shape[i], g.shape.data() + g.lv[i].shape_row);
  }
  for (int i = 0; i < d.n_placed; ++i) {
    const int l = d.pv_logical[i], m = d.pv_mother[i];
    if (l < 0 || l >= d.n_logical || m < VGN_BOOLEAN_OPERAND || m >= d.n_logical || (m == -1 && i != d.world_placed)) {
      err = "placed volume " + std::to_string(i) + " refers to an invalid logical volume";
      return VGN_ERR_ARG;
    }
    g.pv[i].lv     = l;
    g.pv[i].mother = m;
    g.pv[i].xf     = xform_from12(d.pv_transform + 12 * (size_t)i);
    if (m >= 0) {
      g.pv[i].child_id = (int32_t)g.lv[m].daughters.size();
      g.lv[m].daughters.push_back(i);
    }
  }
  if (int rc = link_booleans(g, d, err)) return rc;
  if (g.booleans && g.sections) {
    err = "boolean solids in a geometry with phi or theta sections are not supported";
    return VGN_ERR_UNSUPPORTED;
  }
  for (const HostLV &lv : g.lv)
    if (lv.daughters.size() >= 65535) {
      err = "more than 65534 daughters in one volume";
      return VGN_ERR_UNSUPPORTED;
    }
  // the world must reach every placement exactly once (tree, no cycles)
  {
    std::vector<int> seen(d.n_placed, 0);
    std::function<bool(int, int)> walk = [&](int pv, int level) {
      if (level > kMaxLevels || seen[pv]++) return false;
      for (int c : g.lv[g.pv[pv].lv].daughters)
        if (!walk(c, level + 1)) return false;
      return true;
    };
    if (!walk(g.world_pv, 0)) {
      err = "placement hierarchy is cyclic, shared or deeper than 30 levels";
      return VGN_ERR_UNSUPPORTED;
    }
  }
  g.max_depth = depth_below(g, g.world_pv, 0);

  // daughter boxes and BVHs
  for (size_t i = 0; i < g.lv.size(); ++i) {
    HostLV &lv = g.lv[i];
    if (lv.daughters.empty()) continue;
    lv.aabbs.resize(lv.daughters.size());
    for (size_t k = 0; k < lv.daughters.size(); ++k) lv.aabbs[k] = compute_abbox(g, lv.daughters[k]);
    BVHBuilder(lv.aabbs, lv.bvh).build();
  }
  NavIndexBuilder(g).build();

  // ---- device images ----
  g.pv_rec.assign(g.pv.size(), PVRec());
  for (size_t i = 0; i < g.pv.size(); ++i) {
    PVRec &r = g.pv_rec[i];
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 3; ++k) r.xf.t[k] = g.pv[i].xf.t[k];
    for (int k = 0; k < 9; ++k) r.xf.r[k] = g.pv[i].xf.r[k];
    r.lv        = g.pv[i].lv;
    r.child_id  = g.pv[i].child_id;
    r.xf_flags  = (g.pv[i].xf.has_trans ? kXfTrans : 0) | (g.pv[i].xf.has_rot ? kXfRot : 0);
    r.shape     = g.lv[r.lv].shape;
    r.shape_row = g.lv[r.lv].shape_row;
  }
  // every shape's bounding box, as VUnplacedVolume::ComputeBBox caches it at construction
  g.lv_bbox.assign(6 * g.lv.size(), 0.);
  for (size_t l = 0; l < g.lv.size(); ++l) {
    Vec3 lower, upper;
    shape_extent(g.lv[l].shape, &g.shape[g.lv[l].shape_row], lower, upper);
    const double b[6] = {lower.x, lower.y, lower.z, upper.x, upper.y, upper.z};
    std::copy(b, b + 6, g.lv_bbox.begin() + 6 * l);
  }
  g.lv_rec.assign(g.lv.size(), LVRec());
  g.daughters.clear();
  g.nodes.clear();
  g.prims.clear();
  g.fnodes.clear();
  g.fprims.clear();
  for (size_t i = 0; i < g.lv.size(); ++i) {
    const HostLV &lv = g.lv[i];
    LVRec &r         = g.lv_rec[i];
    std::memset(&r, 0, sizeof(r));
    r.shape         = lv.shape;
    r.shape_row     = lv.shape_row;
    r.nd            = (int32_t)lv.daughters.size();
    r.daughters_off = (int32_t)g.daughters.size();
    g.daughters.insert(g.daughters.end(), lv.daughters.begin(), lv.daughters.end());
    if (lv.daughters.empty()) continue;
    r.nodes_off = (int32_t)g.nodes.size();
    r.n_nodes   = (int32_t)lv.bvh.nodes.size();
    r.prims_off = (int32_t)g.prims.size();
    r.depth     = (uint16_t)lv.bvh.depth;
    for (int d : lv.daughters) r.dtypes |= (uint16_t)(1u << g.lv[g.pv[d].lv].shape);
    for (size_t k = 0; k < lv.bvh.nodes.size(); ++k) {
      NodeRec n;
      FNodeRec f;
      std::memset(&n, 0, sizeof(n));
      const Box3 &b = lv.bvh.nodes[k];
      n.mn[0] = b.mn.x; n.mn[1] = b.mn.y; n.mn[2] = b.mn.z;
      n.mx[0] = b.mx.x; n.mx[1] = b.mx.y; n.mx[2] = b.mx.z;
      n.nchild = lv.bvh.nchild[k];
      n.offset = lv.bvh.offset[k];
      for (int c = 0; c < 3; ++c) {
        f.mn[c] = round_down(n.mn[c]);
        f.mx[c] = round_up(n.mx[c]);
      }
      f.nchild = n.nchild;
      f.offset = n.offset;
      g.nodes.push_back(n);
      g.fnodes.push_back(f);
    }
    // leaf primitives in BVH order: position p holds daughter prim_id[p]
    for (size_t p = 0; p < lv.daughters.size(); ++p) {
      const int prim = lv.bvh.prim_id[p];
      const Box3 &b  = lv.aabbs[prim];
      PrimRec q;
      FPrimRec f;
      std::memset(&q, 0, sizeof(q));
      q.mn[0] = b.mn.x; q.mn[1] = b.mn.y; q.mn[2] = b.mn.z;
      q.mx[0] = b.mx.x; q.mx[1] = b.mx.y; q.mx[2] = b.mx.z;
      q.pv   = lv.daughters[prim];
      q.prim = prim;
      for (int c = 0; c < 3; ++c) {
        f.mn[c] = round_down(q.mn[c]);
        f.mx[c] = round_up(q.mx[c]);
      }
      f.pv   = q.pv;
      f.prim = prim;
      g.prims.push_back(q);
      g.fprims.push_back(f);
    }
  }
  build_interval_images(g);
  return VGN_OK;
}

void set_interval(float *lo, float *hi, double v)
{
  *lo = round_down(v);
  *hi = round_up(v);
}

// Appends the interval SafetyToIn row (geom_types.h irow) of one shape to `out` and
// returns its first pair index, or -1 for shapes without one (Box uses IXForm's
// half-lengths; phi or theta sections and the CutTube are evaluated in FP64).  Each derived value is computed with
// the same FP64 operations as the device's SafetyToIn (host code is built with
// -ffp-contract=off), so its enclosure also encloses the device's double.
static int build_isin_row(int shape, const double *r, std::vector<float> &out)
{
  constexpr double kTolerance = 1e-9, kConeTolerance = 1e-7;  // base/Math.h, ConeStruct
  std::vector<double> v;
  switch (shape) {
  case kTube:  // TubeImplementation.h:912-938; a phi section is evaluated in FP64
    if (r[row::TubeDphi] < 2. * 3.14159265358979323846) return -1;
    v = {r[row::TubeZ], r[row::TubeRmax], r[row::TubeRmin], r[row::TubeRmin] > 0 ? 1. : 0.};
    break;
  case kCone: {  // ConeImplementation.h:368-432, ConeUtilities.h cone radius / safety to the conical surface
    if (r[row::ConeDPhi] < 2. * 3.14159265358979323846) return -1;  // a phi section is evaluated in FP64
    v.assign(irow::kConeRow, 0.);
    v[irow::ConeDz]           = r[row::ConeDz];
    v[irow::ConeMinusConeTol] = -kConeTolerance;
    v[irow::ConeTol]          = kTolerance;
    v[irow::ConeHasRmin]      = (r[row::ConeRmin1] > 0 || r[row::ConeRmin2] > 0) ? 1. : 0.;
    v[irow::ConeOuterConst]   = r[row::ConeOrigRmax1] == r[row::ConeOrigRmax2] ? 1. : 0.;
    v[irow::ConeOuterR]       = r[row::ConeOrigRmax1];
    v[irow::ConeOuterSlope]   = r[row::ConeOuterSlope];
    v[irow::ConeOuterOffset]  = r[row::ConeOuterOffset];
    v[irow::ConeTwoOuterTol]  = 2.0 * r[row::ConeOuterTol];
    v[irow::ConeInnerConst]   = r[row::ConeRmin1] == r[row::ConeRmin2] ? 1. : 0.;
    v[irow::ConeInnerR]       = r[row::ConeRmin1];
    v[irow::ConeInnerSlope]   = r[row::ConeInnerSlope];
    v[irow::ConeInnerOffset]  = r[row::ConeInnerOffset];
    v[irow::ConeTwoInnerTol]  = 2.0 * r[row::ConeInnerTol];
    v[irow::ConeTanRMax]      = r[row::ConeTanRMax];
    v[irow::ConeAvgRmax]      = (r[row::ConeRmax1] + r[row::ConeRmax2]) * 0.5;
    v[irow::ConeInvSecRMax]   = r[row::ConeInvSecRMax];
    v[irow::ConeTanRMin]      = r[row::ConeTanRMin];
    v[irow::ConeAvgRmin]      = (r[row::ConeRmin1] + r[row::ConeRmin2]) * 0.5;
    v[irow::ConeInvSecRMin]   = r[row::ConeInvSecRMin];
    break;
  }
  case kTrd:  // TrdImplementation.h:140-168
    v = {r[row::TrdDz],  r[row::TrdHalfX1plusX2], r[row::TrdFx], r[row::TrdCalfX],
         r[row::TrdDy1] != r[row::TrdDy2] ? 1. : 0., r[row::TrdHalfY1plusY2], r[row::TrdFy], r[row::TrdCalfY],
         r[row::TrdDy1]};
    break;
  case kTrapezoid:  // TrapezoidImplementation.h:341-371 over PlaneShell<4>
    v.assign(r, r + irow::kTrapRow);
    break;
  case kSphere: {  // SphereImplementation.h:388-420, SphereUtilities.h:54-108 (full sphere)
    if (r[row::SphFull] == 0.) return -1;  // phi or theta sections: FP64 only
    const double rmin = r[row::SphRmin], rmax = r[row::SphRmax];
    v = {rmin != 0. ? 1. : 0., rmin, rmax, std::fabs(rmax * (rmax - 2.0 * kTolerance)),
         rmax * (rmax + 2.0 * kTolerance), rmin * (rmin + 2.0 * kTolerance),
         std::fabs(rmin * (rmin - 2.0 * kTolerance))};
    break;
  }
  case kOrb:  // OrbImplementation.h SafetyToIn: |p| - R, with the tolerance shell around R
    v = {r[0], r[0] - kTolerance, r[0] + kTolerance};
    break;
  case kPolycone: {  // PolyconeImplementation.h:381-450 over the sections' (full) cone rows
    const int n = (int)r[row::PconNSec];
    std::vector<float> cones;
    for (int k = 0; k < n; ++k)
      if (build_isin_row(kCone, r + row::pcon_cone(n, k), cones) < 0) return -1;  // phi section
    v = {(double)n, kTolerance};
    for (int k = 0; k <= n; ++k) v.push_back(r[row::PconZs + k]);
    for (int k = 0; k < n; ++k) v.push_back(r[row::pcon_shift(n) + k]);
    const int pos = (int)(out.size() / 2);
    for (double d : v) {
      float lo, hi;
      set_interval(&lo, &hi, d);
      out.push_back(lo);
      out.push_back(hi);
    }
    out.insert(out.end(), cones.begin(), cones.end());
    return pos;
  }
  default: return -1;
  }
  const int pos = (int)(out.size() / 2);
  for (double d : v) {
    float lo, hi;
    set_interval(&lo, &hi, d);
    out.push_back(lo);
    out.push_back(hi);
  }
  return pos;
}

// Interval (FP32) images of the FP64 tables, for the mixed-precision kernels.
void build_interval_images(HostGeometry &g)
{
  auto slab = [](const double *mn, const double *mx, float *mn_lo, float *mn_hi, float *mx_lo, float *mx_hi) {
    for (int c = 0; c < 3; ++c) {
      set_interval(&mn_lo[c], &mn_hi[c], mn[c]);
      set_interval(&mx_lo[c], &mx_hi[c], mx[c]);
    }
  };
  // AABB::Safety (AABB.h:81) uses Center() = 0.5*(max+min) and 0.5*Size() = 0.5*(max-min)
  auto safe = [](const double *mn, const double *mx, ISafe &s) {
    std::memset(&s, 0, sizeof(s));
    for (int c = 0; c < 3; ++c) {
      const double centre = 0.5 * (mx[c] + mn[c]);
      const double half   = 0.5 * (mx[c] - mn[c]);
      set_interval(&s.c_lo[c], &s.c_hi[c], centre);
      set_interval(&s.hs_lo[c], &s.hs_hi[c], half);
    }
  };
  g.inodes.assign(g.nodes.size(), INodeSlab());
  g.inode_safe.assign(g.nodes.size(), ISafe());
  for (size_t i = 0; i < g.nodes.size(); ++i) {
    INodeSlab &n = g.inodes[i];
    std::memset(&n, 0, sizeof(n));
    slab(g.nodes[i].mn, g.nodes[i].mx, n.mn_lo, n.mn_hi, n.mx_lo, n.mx_hi);
    n.nchild = g.nodes[i].nchild;
    n.offset = g.nodes[i].offset;
    safe(g.nodes[i].mn, g.nodes[i].mx, g.inode_safe[i]);
  }
  g.iprims.assign(g.prims.size(), IPrimSlab());
  g.iprim_safe.assign(g.prims.size(), ISafe());
  for (size_t i = 0; i < g.prims.size(); ++i) {
    IPrimSlab &p = g.iprims[i];
    std::memset(&p, 0, sizeof(p));
    slab(g.prims[i].mn, g.prims[i].mx, p.mn_lo, p.mn_hi, p.mx_lo, p.mx_hi);
    p.pv   = g.prims[i].pv;
    p.prim = g.prims[i].prim;
    p.shape = g.lv[g.pv[p.pv].lv].shape;
    safe(g.prims[i].mn, g.prims[i].mx, g.iprim_safe[i]);
  }
  // interval SafetyToIn rows, one per logical volume of a shape that has one
  std::vector<int32_t> lv_isin(g.lv.size(), -1);
  g.isin.clear();
  for (size_t l = 0; l < g.lv.size(); ++l) {
    const int pos = build_isin_row(g.lv[l].shape, &g.shape[g.lv[l].shape_row], g.isin);
    if (pos >= 0) lv_isin[l] = pos;
  }
  g.ixf.assign(g.pv.size(), IXForm());
  for (size_t i = 0; i < g.pv.size(); ++i) {
    IXForm &x = g.ixf[i];
    std::memset(&x, 0, sizeof(x));
    for (int c = 0; c < 3; ++c) set_interval(&x.t_lo[c], &x.t_hi[c], g.pv[i].xf.t[c]);
    for (int c = 0; c < 9; ++c) set_interval(&x.r_lo[c], &x.r_hi[c], g.pv[i].xf.r[c]);
    const HostLV &lv = g.lv[g.pv[i].lv];
    x.shape          = lv.shape;
    x.isin           = lv_isin[g.pv[i].lv];
    if (lv.shape == kBox)
      for (int c = 0; c < 3; ++c) set_interval(&x.h_lo[c], &x.h_hi[c], g.shape[lv.shape_row + c]);
  }
}

}  // namespace vgn
