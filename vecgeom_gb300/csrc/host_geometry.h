// host_geometry.h -- host-side geometry closing for libvgnav.
//
// Turns a vgn_geometry_desc into the flat tables of geom_types.h: shape
// rows, placements, daughter lists, daughter AABBs, SAH BVHs and the
// navigation index table.  Runs once per geometry, on the host, in C++.
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "geom_types.h"

struct vgn_geometry_desc;

namespace vgn {

struct Vec3 {
  double x, y, z;
};

struct HostXForm {
  double t[3];
  double r[9];
  bool identity, has_rot, has_trans;
};

struct Box3 {
  Vec3 mn, mx;
};

struct HostBVH {
  int depth = 0;
  std::vector<int32_t> prim_id, offset, nchild;
  std::vector<Box3> nodes;  // (2 << depth) - 1
};

struct HostLV {
  int32_t shape = 0;
  int32_t shape_row = 0;  // offset into HostGeometry::shape
  std::vector<int32_t> daughters;
  std::vector<Box3> aabbs;  // per daughter, mother frame
  HostBVH bvh;
};

struct HostPV {
  int32_t lv = 0, mother = -1, child_id = 0;
  HostXForm xf;
};

struct HostGeometry {
  std::vector<HostLV> lv;
  std::vector<HostPV> pv;
  std::vector<double> shape;      // shape rows
  std::vector<uint32_t> navind;   // navigation index table
  std::vector<uint32_t> node_start; // bitset over navind words: 1 where a state's record starts
  int32_t world_pv = 0;
  int32_t max_depth = 0;    // deepest level below the world (the world is level 0)
  int32_t cache_depth = 0;  // GeoManager::SetTransformationCacheDepth: 0 = every level's matrix cached

  // flattened device images
  std::vector<PVRec> pv_rec;
  std::vector<LVRec> lv_rec;
  std::vector<int32_t> daughters;
  std::vector<NodeRec> nodes;
  std::vector<PrimRec> prims;
  std::vector<FNodeRec> fnodes;
  std::vector<FPrimRec> fprims;
  std::vector<INodeSlab> inodes;
  std::vector<ISafe> inode_safe;
  std::vector<IPrimSlab> iprims;
  std::vector<ISafe> iprim_safe;
  std::vector<IXForm> ixf;
  std::vector<float> isin;  // interval SafetyToIn rows (geom_types.h irow), (lo, hi) pairs
  std::vector<double> lv_bbox;  // per logical volume: shape Extent, min then max corner (VUnplacedVolume::fBBox)
  bool sections = false;    // some shape has a phi or theta section: needs the `sections` kernel set
  bool booleans = false;    // some shape is a boolean solid: needs the `booleans` kernel set
  // the kernel set for this geometry: 0 full_ranges, 1 sections, 2 booleans (full ranges and booleans)
  int kset() const { return booleans ? 2 : (sections ? 1 : 0); }
};

// Returns 0 on success, a VGN_ERR_* code otherwise (message in err).  `cache_depth` as
// GeoManager::SetTransformationCacheDepth (GeoManager.h:121): navigation-table nodes deeper
// than it carry no cached global matrix (0: all levels cached).
int build_host_geometry(const vgn_geometry_desc &desc, HostGeometry &g, std::string &err, int32_t cache_depth = 0);

// transformation helpers (Transformation3D semantics)
HostXForm xform_from12(const double *a);
void xform_identity(HostXForm &m);
void xform_multiply_from_right(HostXForm &m, const HostXForm &rhs);
Vec3 xform_inverse_transform(const HostXForm &m, const Vec3 &p);

// shape rows: returns 0 / VGN_ERR_* ; appends the row to `shape`
int shape_make_row(int32_t type, const double *params, int32_t n_avail, std::vector<double> &shape, std::string &err);
int shape_param_count(int32_t type, const double *params, int32_t n_avail);
void shape_extent(int32_t type, const double *row, Vec3 &mn, Vec3 &mx);
bool shape_row_has_sections(int32_t type, const double *row);  // a phi or theta section

}  // namespace vgn
