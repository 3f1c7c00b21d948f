// vgref_bvh.cpp -- reads the arrays of a reference BVH (VecGeom/base/BVH.h:364-370).
//
// TEST INFRASTRUCTURE ONLY (part of oracle/_ref/libvgref.so, see vgref.cpp).  The BVH
// keeps fPrimId, fOffset, fNChild, fNodes, fAABBs and fDepth private and has no
// accessor for them; this translation unit alone opens the class's private section
// (after every standard header it needs is already in) so that the tests can compare
// the reference's own trees word for word with the product's and the C oracle's.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define private public
#include "VecGeom/base/BVH.h"
#undef private

using vecgeom::BVH;

extern "C" int vgref_bvh_read(const void *bvhp, int *depth, int *n_nodes, int *n_prims, int *prim_id, int *offset,
                              int *nchild, double *nodes_minmax, double *prims_minmax)
{
  const BVH *b = static_cast<const BVH *>(bvhp);
  // node count of a complete tree of the BVH's depth (source/BVH.cpp:71-73)
  const int nn = (2 << b->fDepth) - 1;
  const int np = (int)b->fLV.GetDaughters().size();
  *depth       = b->fDepth;
  *n_nodes     = nn;
  *n_prims     = np;
  if (prim_id) std::memcpy(prim_id, b->fPrimId, sizeof(int) * (size_t)np);
  if (offset) std::memcpy(offset, b->fOffset, sizeof(int) * (size_t)nn);
  if (nchild) std::memcpy(nchild, b->fNChild, sizeof(int) * (size_t)nn);
  for (int i = 0; nodes_minmax && i < nn; ++i) {
    const auto mn = b->fNodes[i].Min(), mx = b->fNodes[i].Max();
    for (int k = 0; k < 3; ++k) {
      nodes_minmax[6 * i + k]     = mn[k];
      nodes_minmax[6 * i + 3 + k] = mx[k];
    }
  }
  for (int i = 0; prims_minmax && i < np; ++i) {
    const auto mn = b->fAABBs[i].Min(), mx = b->fAABBs[i].Max();
    for (int k = 0; k < 3; ++k) {
      prims_minmax[6 * i + k]     = mn[k];
      prims_minmax[6 * i + 3 + k] = mx[k];
    }
  }
  return 0;
}
