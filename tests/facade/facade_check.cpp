// facade_check.cpp -- checks include/vgnav_vecgeom.hpp against VecGeom's own geometry.
//
// Built by tests/test_vecgeom_facade.py against the reference headers (with the scalar
// VecCore stand-in of oracle/ref/shim), oracle/_ref/libvgref.so (VecGeom's navigation
// sources) and libvgnav.  Reads a flat geometry description, builds it with VecGeom's
// API (vgref_geom_create), exports it with vgnav::ExportGeometry, closes the export with
// libvgnav on the host, and compares the navigation table and every BVH word for word with
// VecGeom's.  Then it installs vgnav::GpuBVHNavigator on the volumes with daughters and
//  - calls a batch method through a vecgeom::VNavigator pointer (with a host-only
//    geometry the library must answer VGN_ERR_ARG, which shows the call reached it);
//  - compares the navigator's scalar calls with VecGeom's BVHNavigator on sample tracks.
// Prints one "key value" line per check.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "VecGeom/management/NavIndexTable.h"
#include "VecGeom/navigation/BVHNavigator.h"
#include "vgnav_vecgeom.hpp"

extern "C" {
int vgref_geom_create(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params, int n_params,
                      int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans, int world_pv,
                      int cache_depth, char *err, int errlen);
int vgref_bvh_info(int lv, int *depth, int *n_nodes, int *n_prims);
int vgref_bvh_arrays(int lv, int *prim_id, int *offset, int *nchild, double *nodes_minmax, double *prims_minmax);
}

using namespace vecgeom;

template <typename T>
static bool read(std::ifstream &f, std::vector<T> &v, size_t n)
{
  v.resize(n);
  return (bool)f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(T)));
}

// words of the reference table that its builder never writes (source/NavIndexTable.cpp:24-67)
static std::vector<bool> pad_words(const uint32_t *t, size_t n)
{
  std::vector<bool> pad(n, false);
  size_t i = 1;
  while (i < n) {
    const uint32_t w = t[i + 2], hasm = (w >> 8) & 0xffu, nd = w >> 16;
    if ((nd + 1) & 1u) pad[i + 3 + nd] = true;
    size_t cur = i + 3 + nd + ((nd + 1) & 1u);
    if (hasm) {
      if (cur % 2) pad[cur++] = true;
      cur += 24;
    }
    i = cur;
  }
  return pad;
}

int main(int argc, char **argv)
{
  if (argc < 2) return 2;
  std::ifstream f(argv[1], std::ios::binary);
  int32_t hdr[4];
  f.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
  const int n_lv = hdr[0], n_pv = hdr[1], n_params = hdr[2], world = hdr[3];
  std::vector<int32_t> lv_shape, lv_off, pv_lv, pv_mother;
  std::vector<double> params, xf;
  if (!read(f, lv_shape, n_lv) || !read(f, lv_off, n_lv) || !read(f, pv_lv, n_pv) || !read(f, pv_mother, n_pv) ||
      !read(f, params, n_params) || !read(f, xf, 12 * (size_t)n_pv))
    return 3;
  char err[256] = {0};
  if (vgref_geom_create(n_lv, lv_shape.data(), lv_off.data(), params.data(), n_params, n_pv, pv_lv.data(),
                        pv_mother.data(), xf.data(), world, 0, err, 256)) {
    std::printf("error %s\n", err);
    return 4;
  }

  // 1. the export describes the geometry it was built from
  const vgnav::ExportedGeometry e = vgnav::ExportGeometry();
  std::printf("export_same_placements %d\n", (int)(e.pv_logical == pv_lv && e.pv_mother == pv_mother &&
                                                    e.pv_transform == xf && e.world_placed == world));
  int same_params = (int)(e.lv_shape == lv_shape && e.params.size() == params.size());
  if (same_params)
    for (size_t i = 0; i < params.size(); ++i)
      if (std::memcmp(&params[i], &e.params[i], sizeof(double))) same_params = 0;
  std::printf("export_same_params %d\n", same_params);
  if (argc > 2) {  // the export, in the input's format
    std::ofstream o(argv[2], std::ios::binary);
    const int32_t h[4] = {(int32_t)e.lv_shape.size(), (int32_t)e.pv_logical.size(), (int32_t)e.params.size(),
                          e.world_placed};
    o.write(reinterpret_cast<const char *>(h), sizeof(h));
    auto put = [&o](const auto &v) { o.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(v[0]))); };
    put(e.lv_shape);
    put(e.lv_param_offset);
    put(e.pv_logical);
    put(e.pv_mother);
    put(e.params);
    put(e.pv_transform);
  }

  // 2. libvgnav closes the export into VecGeom's own tables
  const vgn_geometry_desc d = e.desc();
  vgn_geometry *g           = nullptr;
  if (vgn_geometry_create(&d, VGN_HOST_ONLY, &g) != VGN_OK) {
    std::printf("error %s\n", vgn_last_error());
    return 5;
  }
  const uint32_t *mine = nullptr;
  size_t n_mine        = 0;
  vgn_geometry_navindex(g, &mine, &n_mine);
  const uint32_t *ref  = NavIndexTable::Instance()->GetTable();
  const size_t n_ref   = NavIndexTable::Instance()->GetTableSize() / sizeof(uint32_t);
  const auto pad       = pad_words(ref, n_ref);
  size_t diff          = (n_mine == n_ref + 1) ? 0 : 1;
  for (size_t i = 0; !diff && i < n_ref; ++i)
    if (!pad[i] && mine[i] != ref[i]) ++diff;
  std::printf("navindex_equal %d\n", (int)(diff == 0));
  int bvh_ok = 1, n_bvh = 0;
  for (int lv = 0; lv < n_lv; ++lv) {
    int rd, rn, rp;
    if (vgref_bvh_info(lv, &rd, &rn, &rp)) continue;
    ++n_bvh;
    int32_t md, mn, mp;
    if (vgn_geometry_bvh_info(g, lv, &md, &mn, &mp) != VGN_OK || md != rd || mn != rn || mp != rp) {
      bvh_ok = 0;
      continue;
    }
    std::vector<int> a0(rp), a1(rn), a2(rn), b0(rp), b1(rn), b2(rn);
    std::vector<double> a3(6 * (size_t)rn), a4(6 * (size_t)rp), b3(6 * (size_t)rn), b4(6 * (size_t)rp);
    vgref_bvh_arrays(lv, a0.data(), a1.data(), a2.data(), a3.data(), a4.data());
    vgn_geometry_bvh_arrays(g, lv, b0.data(), b1.data(), b2.data(), b3.data(), b4.data());
    if (a0 != b0 || a1 != b1 || a2 != b2 || std::memcmp(a3.data(), b3.data(), a3.size() * sizeof(double)) ||
        std::memcmp(a4.data(), b4.data(), a4.size() * sizeof(double)))
      bvh_ok = 0;
  }
  std::printf("bvh_equal %d %d\n", bvh_ok, n_bvh);

  // 3. the navigator installed on the volumes, called through VNavigator pointers
  vgnav::GpuBVHNavigator gpu(g, VGN_PRECISION_MIXED, nullptr);
  for (auto &it : GeoManager::Instance().GetLogicalVolumesMap())
    if (it.second->GetDaughters().size()) it.second->SetNavigator(&gpu);
  LogicalVolume const *wl = GeoManager::Instance().GetWorld()->GetLogicalVolume();
  VNavigator const *nav   = wl->GetNavigator();
  std::printf("navigator_name %s\n", nav->GetName());
  const int n = 64;
  std::vector<double> px(n), py(n), pz(n), dx(n), dy(n), dz(n), sl(n, 1.0e4), st(n), sf(n);
  Vector3D<Precision> lo, hi;
  wl->GetUnplacedVolume()->Extent(lo, hi);
  for (int i = 0; i < n; ++i) {  // points spread through the world, directions on a spiral
    const double u = (i + 0.5) / n, phi = 2.399963 * i, z = 1.0 - 2.0 * u, r = std::sqrt(1.0 - z * z);
    px[i] = lo.x() + (hi.x() - lo.x()) * std::fmod(0.618034 * i, 1.0);
    py[i] = lo.y() + (hi.y() - lo.y()) * std::fmod(0.414214 * i + 0.3, 1.0);
    pz[i] = lo.z() + (hi.z() - lo.z()) * u;
    dx[i] = r * std::cos(phi);
    dy[i] = r * std::sin(phi);
    dz[i] = z;
  }
  SOA3D<Precision> pts(px.data(), py.data(), pz.data(), n), dirs(dx.data(), dy.data(), dz.data(), n);
  NavStatePool in(n, GeoManager::Instance().getMaxDepth()), out(n, GeoManager::Instance().getMaxDepth());
  for (int i = 0; i < n; ++i) GlobalLocator::LocateGlobalPoint(GeoManager::Instance().GetWorld(), pts[i], *in[i], true);
  bool calc[n];
  for (int i = 0; i < n; ++i) calc[i] = (i % 2) == 0;
  int code = -1;
  try {
    nav->ComputeStepsAndSafetiesAndPropagatedStates(pts, dirs, sl.data(), in, out, st.data(), calc, sf.data());
    code = 0;
  } catch (vgnav::Error const &x) {
    code = x.code();
  }
  std::printf("batch_call_status %d\n", code);

  // scalar calls: VecGeom's own BVH navigation through the same navigator
  int scalar_same = 1;
  VNavigator const *bvh = BVHNavigator<>::Instance();
  for (int i = 0; i < n; ++i) {
    NavigationState const &s = *in[i];
    if (s.Top() == nullptr || s.Top()->GetLogicalVolume() != wl) continue;
    NavigationState o1, o2;
    const double a = nav->ComputeStepAndPropagatedState(pts[i], dirs[i], sl[i], s, o1);
    const double b = bvh->ComputeStepAndPropagatedState(pts[i], dirs[i], sl[i], s, o2);
    if (std::memcmp(&a, &b, sizeof(double)) || o1.GetNavIndex() != o2.GetNavIndex() ||
        o1.IsOnBoundary() != o2.IsOnBoundary() || o1.GetLastExited() != o2.GetLastExited())
      scalar_same = 0;
  }
  std::printf("scalar_same %d\n", scalar_same);
  vgn_geometry_free(g);
  return 0;
}
