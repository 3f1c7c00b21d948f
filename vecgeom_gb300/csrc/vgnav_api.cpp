// vgnav_api.cpp -- implementation of the C ABI declared in include/vgnav.h.
//
// Owns the device copy of a closed geometry (one flat upload per table,
// instead of the reference's per-object deep copy), validates arguments,
// stages host buffers through a device workspace when the caller passes host
// memory, and maps device-side error bits to status codes.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/vgnav.h"
#include "host_geometry.h"
#include "launch.h"

struct vgn_geometry {
  int device = 0;
  int num_sms = 0;
  vgn::HostGeometry host;
  std::vector<void *> allocations;
  size_t device_bytes = 0;
  uint32_t *d_status  = nullptr;
  vgn::GeomView view{};
  // staging workspace for calls made with host pointers
  std::mutex ws_mutex;
  void *d_ws      = nullptr;
  size_t ws_bytes = 0;
  // step launch configuration per precision form (0 = FP64, 1 = mixed):
  // kernel launch-shape variant and track-binning granularity (0 = no binning)
  int step_variant[2] = {0, 0};
  int sort_kbits[2]   = {0, 0};
  // the safety pass's own visit order: tracks binned by position alone into 2^k cells per
  // axis (0 = the step's order)
  int safety_kbits[2] = {0, 0};
  vgn::BinParams bin{};
  // pipelined staging of host-buffer steps: pieces alternate between two internal streams,
  // each with its own half of the staging workspace and of `d_pipe_sort`
  int staging_chunks      = 0;  // 0 = automatic
  cudaStream_t pipe[2]    = {nullptr, nullptr};
  cudaEvent_t pipe_ev[3]  = {nullptr, nullptr, nullptr};  // fork, join of pipe[0], join of pipe[1]
  uint32_t *d_pipe_sort   = nullptr;
  size_t pipe_sort_words  = 0;
};

// The kernel set a call runs on (HostGeometry::kset): `booleans` when the geometry holds a
// boolean solid, else `sections` when a shape has a phi or theta section, else `full_ranges`
// (the same kernels compiled without the section and boolean code).
#define VGN_KSET_FN(kset, fn) ((kset) == 2 ? vgn::booleans::fn : (kset) == 1 ? vgn::sections::fn : vgn::full_ranges::fn)

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
  return fail(VGN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

class DeviceGuard {
public:
  explicit DeviceGuard(int dev)
  {
    if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
    if (prev_ != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard()
  {
    if (prev_ >= 0) cudaSetDevice(prev_);
  }

private:
  int prev_ = -1;
};

template <typename T>
int upload(vgn_geometry *g, const std::vector<T> &v, const T **dst)
{
  if (v.empty()) {
    *dst = nullptr;
    return VGN_OK;
  }
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, v.size() * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(geometry table)");
  g->allocations.push_back(p);
  g->device_bytes += v.size() * sizeof(T);
  e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(geometry table)");
  *dst = static_cast<const T *>(p);
  return VGN_OK;
}

// true when every non-null pointer is device-accessible, false when all are host
// memory; -1 on a mix.
int classify(std::initializer_list<const void *> ptrs)
{
  int kind = -2;
  for (const void *p : ptrs) {
    if (!p) continue;
    cudaPointerAttributes attr;
    int k = 0;
    if (cudaPointerGetAttributes(&attr, p) == cudaSuccess)
      k = (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) ? 1 : 0;
    else
      cudaGetLastError();
    if (kind == -2)
      kind = k;
    else if (kind != k)
      return -1;
  }
  return kind < 0 ? 0 : kind;
}

int check_status(const vgn_geometry *g, cudaStream_t s)
{
  uint32_t st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, g->d_status, sizeof(st), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "status readback");
  if (st) {
    cudaMemsetAsync(g->d_status, 0, sizeof(uint32_t), s);
    cudaStreamSynchronize(s);
    if (st & vgn::kErrStack) return fail(VGN_ERR_STACK, "BVH traversal stack overflow on the device");
    if (st & vgn::kErrRelocate) return fail(VGN_ERR_RELOCATE, "relocation exceeded the geometry depth bound");
    if (st & vgn::kErrState) return fail(VGN_ERR_STATE, "input navigation state outside the navigation table");
  }
  return VGN_OK;
}

void *workspace(vgn_geometry *g, size_t bytes)
{
  if (bytes <= g->ws_bytes) return g->d_ws;
  if (g->d_ws) cudaFree(g->d_ws);
  g->d_ws     = nullptr;
  g->ws_bytes = 0;
  if (cudaMalloc(&g->d_ws, bytes) != cudaSuccess) {
    cudaGetLastError();
    g->d_ws = nullptr;
    return nullptr;
  }
  g->ws_bytes = bytes;
  return g->d_ws;
}

int max_blocks(const vgn_geometry *g) { return g->num_sms > 0 ? g->num_sms * 32 : 4096; }

// Per-call device scratch (track binning) comes from a stream-ordered memory pool that the
// library creates once per device: an allocation belongs to the stream of the call that made
// it and is released in that stream's order, so calls on different streams (or threads) never
// share scratch.  The pool keeps released blocks (release threshold = no limit), so steady
// calls of one size allocate nothing new; the blocks stay with the process until it exits.
cudaError_t pool_alloc(int device, size_t bytes, cudaStream_t s, void **p)
{
  static std::mutex m;
  static std::vector<cudaMemPool_t> pools;
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lock(m);
    if ((int)pools.size() <= device) pools.resize((size_t)device + 1, nullptr);
    if (!pools[(size_t)device]) {
      cudaMemPoolProps props{};
      props.allocType     = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id   = device;
      cudaError_t e       = cudaMemPoolCreate(&pools[(size_t)device], &props);
      if (e != cudaSuccess) {
        pools[(size_t)device] = nullptr;
        return e;
      }
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pools[(size_t)device], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = pools[(size_t)device];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// Enqueue one step batch with the geometry's launch configuration: optional
// track binning (counting sort into a visit permutation), then the step kernel.
// `scratch` (bin_scratch_words(n, kbits) + n words) replaces the geometry's shared
// binning scratch, for batches staged on the internal streams.
int enqueue_step(vgn_geometry *g, vgn::StepArgs a, bool mixed, cudaStream_t s, uint32_t *scratch = nullptr)
{
  const int m     = mixed ? 1 : 0;
  const int kbits = g->sort_kbits[m];
  a.perm          = nullptr;
  if (kbits > 0 && a.n <= (int64_t)UINT32_MAX && scratch) {
    vgn::BinParams b = g->bin;
    b.kbits          = kbits;
    for (int k = 0; k < 3; ++k) b.scale[k] = g->bin.scale[k] * (float)(1 << kbits);
    uint32_t *perm = scratch + vgn::bin_scratch_words(a.n, kbits);
    cudaError_t e  = vgn::launch_bin_tracks(a.n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, b, scratch, perm,
                                            max_blocks(g), s);
    if (e != cudaSuccess) return cuda_fail(e, "track binning launch");
    a.perm = perm;
  } else if (a.n <= (int64_t)UINT32_MAX) {  // the visit permutations hold 32-bit track indices
    const int ks = a.safety ? g->safety_kbits[m] : 0;
    if (kbits > 0 || ks > 0) {
      // keys and histogram (reused by the two binnings in stream order), then the orders;
      // stream-ordered scratch of this call alone, so calls on other streams never share it
      size_t head = kbits > 0 ? vgn::bin_scratch_words(a.n, kbits) : 0;
      if (ks > 0 && vgn::bin_scratch_words(a.n, ks) > head) head = vgn::bin_scratch_words(a.n, ks);
      const size_t need = head + (size_t)a.n * ((kbits > 0 ? 1 : 0) + (ks > 0 ? 1 : 0));
      uint32_t *buf = nullptr;
      if (pool_alloc(g->device, need * sizeof(uint32_t), s, reinterpret_cast<void **>(&buf)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VGN_ERR_NOMEM, "track-binning scratch allocation failed");
      }
      uint32_t *next = buf + head;
      cudaError_t e  = cudaSuccess;
      if (kbits > 0) {  // the step's order: direction octant, then position
        vgn::BinParams b = g->bin;
        b.kbits          = kbits;
        for (int k = 0; k < 3; ++k) b.scale[k] = g->bin.scale[k] * (float)(1 << kbits);
        e      = vgn::launch_bin_tracks(a.n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, b, buf, next, max_blocks(g), s);
        a.perm = next;
        next += a.n;
      }
      if (e == cudaSuccess && ks > 0) {  // the safety pass's order: position alone
        vgn::BinParams b = g->bin;
        b.kbits          = ks;
        b.octants        = 0;
        for (int k = 0; k < 3; ++k) b.scale[k] = g->bin.scale[k] * (float)(1 << ks);
        e             = vgn::launch_bin_tracks(a.n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, b, buf, next, max_blocks(g), s);
        a.perm_safety = next;
      }
      if (e == cudaSuccess) e = VGN_KSET_FN(g->host.kset(), launch_step)(g->view, a, mixed, g->step_variant[m], s);
      cudaFreeAsync(buf, s);
      return e == cudaSuccess ? VGN_OK : cuda_fail(e, "binned step launch");
    }
  }
  cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_step)(g->view, a, mixed, g->step_variant[m], s);
  return e == cudaSuccess ? VGN_OK : cuda_fail(e, "step kernel launch");
}

// bump allocator over the staging workspace (256-byte aligned sub-buffers)
struct Carve {
  char *base;
  size_t off = 0;
  template <typename T>
  T *take(size_t count)
  {
    T *p = reinterpret_cast<T *>(base + off);
    off += (count * sizeof(T) + 255) & ~size_t(255);
    return p;
  }
};

size_t carve_bytes(std::initializer_list<size_t> sizes)
{
  size_t b = 0;
  for (size_t s : sizes) b += (s + 255) & ~size_t(255);
  return b;
}

}  // namespace

extern "C" {

const char *vgn_last_error(void) { return g_last_error.c_str(); }

const char *vgn_version(void) { return "vgnav-gb300 0.1 (sm_103a)"; }

int vgn_geometry_create(const vgn_geometry_desc *desc, int device, vgn_geometry **out)
{
  return vgn_geometry_create_with_cache_depth(desc, device, 0, out);
}

int vgn_geometry_create_with_cache_depth(const vgn_geometry_desc *desc, int device, int32_t cache_depth,
                                         vgn_geometry **out)
{
  if (!desc || !out) return fail(VGN_ERR_ARG, "null argument");
  *out = nullptr;
  vgn_geometry *g = new (std::nothrow) vgn_geometry();
  if (!g) return fail(VGN_ERR_NOMEM, "host allocation failed");
  std::string err;
  int rc = vgn::build_host_geometry(*desc, g->host, err, cache_depth);
  if (rc) {
    delete g;
    return fail(rc, err);
  }
  g->device = device;
  if (device == VGN_HOST_ONLY) {  // closed on the host, nothing uploaded
    *out = g;
    return VGN_OK;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "cudaGetDeviceCount");
  }
  if (device < 0 || device >= ndev) {
    delete g;
    return fail(VGN_ERR_ARG, "device index out of range");
  }
  DeviceGuard guard(device);
  cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
  vgn::GeomView &v = g->view;
  const vgn::HostGeometry &h = g->host;
  if ((rc = upload(g, h.navind, &v.navind)) || (rc = upload(g, h.node_start, &v.node_start)) || (rc = upload(g, h.pv_rec, &v.pv)) || (rc = upload(g, h.lv_rec, &v.lv)) ||
      (rc = upload(g, h.daughters, &v.daughters)) || (rc = upload(g, h.nodes, &v.nodes)) ||
      (rc = upload(g, h.prims, &v.prims)) || (rc = upload(g, h.fnodes, &v.fnodes)) ||
      (rc = upload(g, h.fprims, &v.fprims)) || (rc = upload(g, h.shape, &v.shape)) ||
      (rc = upload(g, h.inodes, &v.inodes)) || (rc = upload(g, h.inode_safe, &v.inode_safe)) ||
      (rc = upload(g, h.iprims, &v.iprims)) || (rc = upload(g, h.iprim_safe, &v.iprim_safe)) ||
      (rc = upload(g, h.ixf, &v.ixf)) || (rc = upload(g, h.isin, &v.isin)) || (rc = upload(g, h.lv_bbox, &v.lv_bbox))) {
    vgn_geometry_free(g);
    return rc;
  }
  e = cudaMalloc(&g->d_status, sizeof(uint32_t));
  if (e != cudaSuccess) {
    vgn_geometry_free(g);
    return cuda_fail(e, "cudaMalloc(status)");
  }
  cudaMemset(g->d_status, 0, sizeof(uint32_t));
  v.status       = g->d_status;
  v.navind_words = (uint32_t)h.navind.size();
  v.n_pv         = (int32_t)h.pv.size();
  v.n_lv         = (int32_t)h.lv.size();
  v.world_pv     = h.world_pv;
  v.max_depth    = h.max_depth;
  v.stack_limit  = vgn::kStackSize;
  v.level_limit  = vgn::kMaxLevels;
  {  // world bounding box for track binning
    const vgn::HostLV &wl = h.lv[h.pv[h.world_pv].lv];
    vgn::Vec3 mn, mx;
    vgn::shape_extent(wl.shape, &h.shape[wl.shape_row], mn, mx);
    const double lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    for (int k = 0; k < 3; ++k) {
      g->bin.lo[k]    = (float)lo[k];
      g->bin.scale[k] = hi[k] > lo[k] ? (float)(1.0 / (hi[k] - lo[k])) : 0.f;
    }
  }
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    vgn_geometry_free(g);
    return cuda_fail(e, "geometry upload");
  }
  *out = g;
  return VGN_OK;
}

int vgn_geometry_free(vgn_geometry *g)
{
  if (!g) return VGN_OK;
  if (g->device != VGN_HOST_ONLY) {
    DeviceGuard guard(g->device);
    for (void *p : g->allocations) cudaFree(p);
    if (g->d_status) cudaFree(g->d_status);
    if (g->d_ws) cudaFree(g->d_ws);
    if (g->d_pipe_sort) cudaFree(g->d_pipe_sort);
    for (cudaStream_t ps : g->pipe)
      if (ps) cudaStreamDestroy(ps);
    for (cudaEvent_t ev : g->pipe_ev)
      if (ev) cudaEventDestroy(ev);
  }
  delete g;
  return VGN_OK;
}

int vgn_geometry_navindex(const vgn_geometry *g, const uint32_t **table, size_t *n_words)
{
  if (!g || !table || !n_words) return fail(VGN_ERR_ARG, "null argument");
  *table   = g->host.navind.data();
  *n_words = g->host.navind.size();
  return VGN_OK;
}

int vgn_geometry_bvh_info(const vgn_geometry *g, int32_t lv, int32_t *depth, int32_t *n_nodes, int32_t *n_prims)
{
  if (!g || lv < 0 || lv >= (int32_t)g->host.lv.size()) return fail(VGN_ERR_ARG, "bad logical volume");
  const vgn::HostLV &l = g->host.lv[lv];
  if (l.daughters.empty()) return fail(VGN_ERR_ARG, "logical volume has no daughters");
  if (depth) *depth = l.bvh.depth;
  if (n_nodes) *n_nodes = (int32_t)l.bvh.nodes.size();
  if (n_prims) *n_prims = (int32_t)l.daughters.size();
  return VGN_OK;
}

int vgn_geometry_bvh_arrays(const vgn_geometry *g, int32_t lv, int32_t *prim_id, int32_t *offset, int32_t *nchild,
                            double *nodes_minmax, double *prims_minmax)
{
  if (!g || lv < 0 || lv >= (int32_t)g->host.lv.size()) return fail(VGN_ERR_ARG, "bad logical volume");
  const vgn::HostLV &l = g->host.lv[lv];
  if (l.daughters.empty()) return fail(VGN_ERR_ARG, "logical volume has no daughters");
  if (prim_id) std::memcpy(prim_id, l.bvh.prim_id.data(), l.bvh.prim_id.size() * sizeof(int32_t));
  if (offset) std::memcpy(offset, l.bvh.offset.data(), l.bvh.offset.size() * sizeof(int32_t));
  if (nchild) std::memcpy(nchild, l.bvh.nchild.data(), l.bvh.nchild.size() * sizeof(int32_t));
  if (nodes_minmax)
    for (size_t i = 0; i < l.bvh.nodes.size(); ++i) std::memcpy(nodes_minmax + 6 * i, &l.bvh.nodes[i], 6 * sizeof(double));
  if (prims_minmax)
    for (size_t i = 0; i < l.aabbs.size(); ++i) std::memcpy(prims_minmax + 6 * i, &l.aabbs[i], 6 * sizeof(double));
  return VGN_OK;
}

int vgn_geometry_device_bytes(const vgn_geometry *g, size_t *bytes)
{
  if (!g || !bytes) return fail(VGN_ERR_ARG, "null argument");
  *bytes = g->device_bytes;
  return VGN_OK;
}

namespace {

// the two internal streams and three events of the staged paths, created on first use
int ensure_pipe(vgn_geometry *g)
{
  if (g->pipe[0]) return VGN_OK;
  for (int k = 0; k < 2; ++k)
    if (cudaStreamCreateWithFlags(&g->pipe[k], cudaStreamNonBlocking) != cudaSuccess)
      return cuda_fail(cudaGetLastError(), "staging stream creation");
  for (int k = 0; k < 3; ++k)
    if (cudaEventCreateWithFlags(&g->pipe_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return cuda_fail(cudaGetLastError(), "staging event creation");
  return VGN_OK;
}

// Host buffers, one piece, with safeties: the safety pass needs only the positions and the
// states, so the directions and step limits are copied on an internal stream while it runs,
// and the safeties are copied back on that stream while the step kernel runs.  Same kernels,
// orders and results as the staged call without the overlap.  Called with ws_mutex held.
int staged_step_overlap(vgn_geometry *g, vgn::StepArgs a, const double *const src[7], const vgn_state *in,
                        vgn_state *out, double *step, double *safety, bool mixed, cudaStream_t s)
{
  const int64_t n = a.n;
  const size_t nd = (size_t)n * sizeof(double), ns = (size_t)n * sizeof(vgn_state);
  void *ws        = workspace(g, carve_bytes({nd, nd, nd, nd, nd, nd, nd, ns, ns, nd, nd}));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  if (int rc = ensure_pipe(g)) return rc;
  Carve c{static_cast<char *>(ws)};
  double *b[7];
  for (int k = 0; k < 7; ++k) b[k] = c.take<double>(n);
  vgn_state *din = c.take<vgn_state>(n), *dout = c.take<vgn_state>(n);
  double *dstep = c.take<double>(n), *dsaf = c.take<double>(n);
  const int m = mixed ? 1 : 0, kbits = g->sort_kbits[m], ks = g->safety_kbits[m];
  cudaStream_t ps = g->pipe[0];
  cudaError_t e   = cudaEventRecord(g->pipe_ev[0], s);  // the side stream follows the caller's prior work
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ps, g->pipe_ev[0], 0);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k], nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, ns, cudaMemcpyHostToDevice, s);
  for (int k = 3; k < 7 && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k], nd, cudaMemcpyHostToDevice, ps);
  if (e == cudaSuccess) e = cudaEventRecord(g->pipe_ev[1], ps);  // directions and step limits are in
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  a.px = b[0]; a.py = b[1]; a.pz = b[2]; a.dx = b[3]; a.dy = b[4]; a.dz = b[5]; a.slimit = b[6];
  a.in = din; a.out = dout; a.step = dstep; a.safety = dsaf; a.perm = nullptr; a.perm_safety = nullptr;
  // binning scratch: keys and histogram shared by the two binnings in stream order, then the orders
  size_t head = kbits > 0 ? vgn::bin_scratch_words(n, kbits) : 0;
  if (ks > 0 && vgn::bin_scratch_words(n, ks) > head) head = vgn::bin_scratch_words(n, ks);
  const size_t need = head + (size_t)n * ((kbits > 0 ? 1 : 0) + (ks > 0 ? 1 : 0));
  uint32_t *buf     = nullptr;
  if (need > 0 && pool_alloc(g->device, need * sizeof(uint32_t), s, reinterpret_cast<void **>(&buf)) != cudaSuccess) {
    cudaGetLastError();
    return fail(VGN_ERR_NOMEM, "track-binning scratch allocation failed");
  }
  uint32_t *next = buf + head;
  if (ks > 0) {  // the safety pass's order: position alone (the directions are not read)
    vgn::BinParams bp = g->bin;
    bp.kbits          = ks;
    bp.octants        = 0;
    for (int k = 0; k < 3; ++k) bp.scale[k] = g->bin.scale[k] * (float)(1 << ks);
    e             = vgn::launch_bin_tracks(n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, bp, buf, next, max_blocks(g), s);
    a.perm_safety = next;
    next += n;
  }
  if (e == cudaSuccess) e = VGN_KSET_FN(g->host.kset(), launch_safety_only)(g->view, a, mixed, s);
  if (e == cudaSuccess) e = cudaEventRecord(g->pipe_ev[2], s);  // safeties are final
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g->pipe_ev[1], 0);
  if (e == cudaSuccess && kbits > 0) {  // the step's order: direction octant, then position
    vgn::BinParams bp = g->bin;
    bp.kbits          = kbits;
    for (int k = 0; k < 3; ++k) bp.scale[k] = g->bin.scale[k] * (float)(1 << kbits);
    e      = vgn::launch_bin_tracks(n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, bp, buf, next, max_blocks(g), s);
    a.perm = next;
  }
  vgn::StepArgs st = a;
  st.safety        = nullptr;  // the step kernel alone
  if (e == cudaSuccess) e = VGN_KSET_FN(g->host.kset(), launch_step)(g->view, st, mixed, g->step_variant[m], s);
  if (buf) cudaFreeAsync(buf, s);
  if (e != cudaSuccess) return cuda_fail(e, "overlapped step launch");
  e = cudaStreamWaitEvent(ps, g->pipe_ev[2], 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(safety, dsaf, nd, cudaMemcpyDeviceToHost, ps);
  if (e == cudaSuccess) e = cudaEventRecord(g->pipe_ev[1], ps);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, ns, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(step, dstep, nd, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g->pipe_ev[1], 0);  // join the side stream
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

// A host-buffer step in `nchunk` pieces: piece i is copied in, binned, stepped and copied out
// on internal stream i % 2, so the copies of one piece overlap the kernels of the other.
// Tracks are independent, so the results do not depend on the split.  Called with
// ws_mutex held; `s` is forked to the two streams and joins them again.
int staged_step_pipelined(vgn_geometry *g, int64_t n, const double *const src[7], const vgn_state *in,
                          vgn_state *out, double *step, double *safety, bool mixed, int reloc, int nchunk,
                          cudaStream_t s)
{
  const int64_t cn = (n + nchunk - 1) / nchunk;
  const size_t nd = (size_t)cn * sizeof(double), ns = (size_t)cn * sizeof(vgn_state);
  const size_t half = carve_bytes({nd, nd, nd, nd, nd, nd, nd, ns, ns, nd, nd});
  char *ws          = static_cast<char *>(workspace(g, 2 * half));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  const int kbits         = g->sort_kbits[mixed ? 1 : 0];
  const size_t sort_words = kbits > 0 ? vgn::bin_scratch_words(cn, kbits) + (size_t)cn : 0;
  if (2 * sort_words > g->pipe_sort_words) {
    if (g->d_pipe_sort) cudaFree(g->d_pipe_sort);
    g->d_pipe_sort     = nullptr;
    g->pipe_sort_words = 0;
    if (cudaMalloc(&g->d_pipe_sort, 2 * sort_words * sizeof(uint32_t)) != cudaSuccess) {
      cudaGetLastError();
      g->d_pipe_sort = nullptr;
      return fail(VGN_ERR_NOMEM, "staging binning scratch allocation failed");
    }
    g->pipe_sort_words = 2 * sort_words;
  }
  if (int rc = ensure_pipe(g)) return rc;
  cudaError_t e = cudaEventRecord(g->pipe_ev[0], s);
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(g->pipe[k], g->pipe_ev[0], 0);
  if (e != cudaSuccess) return cuda_fail(e, "staging fork");
  int rc = VGN_OK;
  for (int i = 0; i < nchunk && rc == VGN_OK; ++i) {
    const int64_t off = (int64_t)i * cn, m = n - off < cn ? n - off : cn;
    if (m <= 0) break;
    const int j       = i & 1;
    cudaStream_t ps   = g->pipe[j];
    const size_t md = (size_t)m * sizeof(double), ms = (size_t)m * sizeof(vgn_state);
    Carve c{ws + j * half};
    double *b[7];
    for (int k = 0; k < 7; ++k) b[k] = c.take<double>(cn);
    vgn_state *din = c.take<vgn_state>(cn), *dout = c.take<vgn_state>(cn);
    double *dstep = c.take<double>(cn), *dsaf = c.take<double>(cn);
    for (int k = 0; k < 7 && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k] + off, md, cudaMemcpyHostToDevice, ps);
    if (e == cudaSuccess) e = cudaMemcpyAsync(din, in + off, ms, cudaMemcpyHostToDevice, ps);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "host to device copy");
      break;
    }
    vgn::StepArgs a{};
    a.n = m;
    a.reloc = reloc;
    a.max_blocks = max_blocks(g);
    a.px = b[0]; a.py = b[1]; a.pz = b[2]; a.dx = b[3]; a.dy = b[4]; a.dz = b[5]; a.slimit = b[6];
    a.in = din; a.out = dout; a.step = dstep; a.safety = safety ? dsaf : nullptr;
    rc = enqueue_step(g, a, mixed, ps, sort_words ? g->d_pipe_sort + j * sort_words : nullptr);
    if (rc != VGN_OK) break;
    e = cudaMemcpyAsync(out + off, dout, ms, cudaMemcpyDeviceToHost, ps);
    if (e == cudaSuccess) e = cudaMemcpyAsync(step + off, dstep, md, cudaMemcpyDeviceToHost, ps);
    if (e == cudaSuccess && safety) e = cudaMemcpyAsync(safety + off, dsaf, md, cudaMemcpyDeviceToHost, ps);
    if (e != cudaSuccess) rc = cuda_fail(e, "device to host copy");
  }
  // join both streams back into the caller's stream, also after an error
  for (int k = 0; k < 2; ++k) {
    cudaEventRecord(g->pipe_ev[1 + k], g->pipe[k]);
    cudaStreamWaitEvent(s, g->pipe_ev[1 + k], 0);
  }
  if (rc != VGN_OK) return rc;
  return check_status(g, s);
}

}  // namespace

int vgn_compute_step_batch(const vgn_geometry *gc, int64_t n, const double *px, const double *py, const double *pz,
                           const double *dx, const double *dy, const double *dz, const double *step_limit,
                           const vgn_state *in, vgn_state *out, double *step, double *safety, int flags, void *stream)
{
  vgn_geometry *g = const_cast<vgn_geometry *>(gc);
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n == 0) return VGN_OK;
  if (!px || !py || !pz || !dx || !dy || !dz || !step_limit || !in || !out || !step)
    return fail(VGN_ERR_ARG, "null array argument");
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  DeviceGuard guard(g->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int kind = classify({px, py, pz, dx, dy, dz, step_limit, in, out, step, safety});
  if (kind < 0) return fail(VGN_ERR_ARG, "mix of host and device pointers");
  vgn::StepArgs a{};
  a.n          = n;
  a.reloc      = (flags & VGN_NO_RELOCATE) ? 0 : 1;
  a.max_blocks = max_blocks(g);
  if (kind == 1) {
    a.px = px; a.py = py; a.pz = pz; a.dx = dx; a.dy = dy; a.dz = dz; a.slimit = step_limit;
    a.in = in; a.out = out; a.step = step; a.safety = safety;
    return enqueue_step(g, a, mixed, s);
  }
  // host buffers: stage through the device workspace, in pipelined pieces for large batches
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  // automatic = one piece: on a GB300 the copies of a 2^22-track batch take ~2 ms against
  // ~22 ms of kernels, and every piece pays the binning scan again (measured: 2 pieces 5 %
  // slower end to end, 8 pieces 23 % slower)
  const int nchunk = g->staging_chunks > 0 ? g->staging_chunks : 1;
  if (nchunk > 1 && n >= nchunk) {
    const double *src[7] = {px, py, pz, dx, dy, dz, step_limit};
    return staged_step_pipelined(g, n, src, in, out, step, safety, mixed, a.reloc, nchunk, s);
  }
  if (safety && n >= (1 << 16) && n <= (int64_t)UINT32_MAX) {
    const double *src[7] = {px, py, pz, dx, dy, dz, step_limit};
    return staged_step_overlap(g, a, src, in, out, step, safety, mixed, s);
  }
  const size_t nd = (size_t)n * sizeof(double), ns = (size_t)n * sizeof(vgn_state);
  const size_t bytes = carve_bytes({nd, nd, nd, nd, nd, nd, nd, ns, ns, nd, nd});
  void *ws = workspace(g, bytes);
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  Carve c{static_cast<char *>(ws)};
  double *b[7];
  for (int k = 0; k < 7; ++k) b[k] = c.take<double>(n);
  vgn_state *din = c.take<vgn_state>(n), *dout = c.take<vgn_state>(n);
  double *dstep = c.take<double>(n), *dsaf = c.take<double>(n);
  const double *src[7] = {px, py, pz, dx, dy, dz, step_limit};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 7 && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k], nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, ns, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  a.px = b[0]; a.py = b[1]; a.pz = b[2]; a.dx = b[3]; a.dy = b[4]; a.dz = b[5]; a.slimit = b[6];
  a.in = din; a.out = dout; a.step = dstep; a.safety = safety ? dsaf : nullptr;
  const int rc = enqueue_step(g, a, mixed, s);
  if (rc != VGN_OK) return rc;
  e = cudaMemcpyAsync(out, dout, ns, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(step, dstep, nd, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && safety) e = cudaMemcpyAsync(safety, dsaf, nd, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

int vgn_step_and_next_volume(const vgn_geometry *g, int64_t n, const double *px, const double *py, const double *pz,
                             const double *dx, const double *dy, const double *dz, const double *step_limit,
                             const vgn_state *in, vgn_state *out, double *step, double *safety, int flags,
                             void *stream)
{
  return vgn_compute_step_batch(g, n, px, py, pz, dx, dy, dz, step_limit, in, out, step, safety, flags, stream);
}

int vgn_compute_safety_batch(const vgn_geometry *gc, int64_t n, const double *px, const double *py, const double *pz,
                             const vgn_state *in, double *safety, int flags, void *stream)
{
  vgn_geometry *g = const_cast<vgn_geometry *>(gc);
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n == 0) return VGN_OK;
  if (!px || !py || !pz || !in || !safety) return fail(VGN_ERR_ARG, "null array argument");
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  DeviceGuard guard(g->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int kind = classify({px, py, pz, in, safety});
  if (kind < 0) return fail(VGN_ERR_ARG, "mix of host and device pointers");
  if (kind == 1) {
    cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_safety)(g->view, n, px, py, pz, in, safety, mixed, max_blocks(g), s);
    return e == cudaSuccess ? VGN_OK : cuda_fail(e, "safety kernel launch");
  }
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  const size_t nd = (size_t)n * sizeof(double), ns = (size_t)n * sizeof(vgn_state);
  void *ws = workspace(g, carve_bytes({nd, nd, nd, ns, nd}));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  Carve c{static_cast<char *>(ws)};
  double *bx = c.take<double>(n), *by = c.take<double>(n), *bz = c.take<double>(n);
  vgn_state *din = c.take<vgn_state>(n);
  double *dsaf   = c.take<double>(n);
  cudaError_t e  = cudaMemcpyAsync(bx, px, nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(by, py, nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bz, pz, nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, ns, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  e = VGN_KSET_FN(g->host.kset(), launch_safety)(g->view, n, bx, by, bz, din, dsaf, mixed, max_blocks(g), s);
  if (e != cudaSuccess) return cuda_fail(e, "safety kernel launch");
  e = cudaMemcpyAsync(safety, dsaf, nd, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

int vgn_locate_batch(const vgn_geometry *gc, int64_t n, const double *px, const double *py, const double *pz,
                     vgn_state *out, int flags, void *stream)
{
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  vgn_geometry *g = const_cast<vgn_geometry *>(gc);
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n == 0) return VGN_OK;
  if (!px || !py || !pz || !out) return fail(VGN_ERR_ARG, "null array argument");
  DeviceGuard guard(g->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int kind = classify({px, py, pz, out});
  if (kind < 0) return fail(VGN_ERR_ARG, "mix of host and device pointers");
  if (kind == 1) {
    cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_locate)(g->view, n, px, py, pz, out, mixed, max_blocks(g), s);
    return e == cudaSuccess ? VGN_OK : cuda_fail(e, "locate kernel launch");
  }
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  const size_t nd = (size_t)n * sizeof(double), ns = (size_t)n * sizeof(vgn_state);
  void *ws = workspace(g, carve_bytes({nd, nd, nd, ns}));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  Carve c{static_cast<char *>(ws)};
  double *bx = c.take<double>(n), *by = c.take<double>(n), *bz = c.take<double>(n);
  vgn_state *dout = c.take<vgn_state>(n);
  cudaError_t e   = cudaMemcpyAsync(bx, px, nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(by, py, nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bz, pz, nd, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  e = VGN_KSET_FN(g->host.kset(), launch_locate)(g->view, n, bx, by, bz, dout, mixed, max_blocks(g), s);
  if (e != cudaSuccess) return cuda_fail(e, "locate kernel launch");
  e = cudaMemcpyAsync(out, dout, ns, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

int vgn_approach_next_daughter_batch(const vgn_geometry *gc, int64_t n, const int32_t *lv, const double *px,
                                     const double *py, const double *pz, const double *dx, const double *dy,
                                     const double *dz, const int32_t *last_pv, double *step, void *stream)
{
  vgn_geometry *g = const_cast<vgn_geometry *>(gc);
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n == 0) return VGN_OK;
  if (!lv || !px || !py || !pz || !dx || !dy || !dz || !step) return fail(VGN_ERR_ARG, "null array argument");
  DeviceGuard guard(g->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int kind = last_pv ? classify({lv, px, py, pz, dx, dy, dz, last_pv, step})
                           : classify({lv, px, py, pz, dx, dy, dz, step});
  if (kind < 0) return fail(VGN_ERR_ARG, "mix of host and device pointers");
  if (kind == 1) {
    cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_approach)(g->view, n, lv, px, py, pz, dx, dy, dz, last_pv,
                                                                   step, max_blocks(g), s);
    return e == cudaSuccess ? VGN_OK : cuda_fail(e, "approach kernel launch");
  }
  // host buffers: the volume ids are checked here, before anything is copied
  const int32_t n_lv = (int32_t)g->host.lv.size(), n_pv = (int32_t)g->host.pv.size();
  for (int64_t i = 0; i < n; ++i) {
    if (lv[i] < 0 || lv[i] >= n_lv || g->host.lv[lv[i]].daughters.empty())
      return fail(VGN_ERR_ARG, "logical volume out of range or without daughters");
    if (last_pv && (last_pv[i] < -1 || last_pv[i] >= n_pv)) return fail(VGN_ERR_ARG, "last placed volume out of range");
  }
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  const size_t nd = (size_t)n * sizeof(double), ni = (size_t)n * sizeof(int32_t);
  void *ws = workspace(g, carve_bytes({nd, nd, nd, nd, nd, nd, nd, ni, ni}));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  Carve c{static_cast<char *>(ws)};
  double *b[7];
  for (auto &p : b) p = c.take<double>(n);
  int32_t *dlv = c.take<int32_t>(n), *dlast = c.take<int32_t>(n);
  const double *src[7] = {px, py, pz, dx, dy, dz, step};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 7 && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k], nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dlv, lv, ni, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && last_pv) e = cudaMemcpyAsync(dlast, last_pv, ni, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  e = VGN_KSET_FN(g->host.kset(), launch_approach)(g->view, n, dlv, b[0], b[1], b[2], b[3], b[4], b[5],
                                                     last_pv ? dlast : nullptr, b[6], max_blocks(g), s);
  if (e != cudaSuccess) return cuda_fail(e, "approach kernel launch");
  e = cudaMemcpyAsync(step, b[6], nd, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

// a boolean (or an operand of it) is a union
static bool boolean_has_union(const vgn::HostGeometry &h, int32_t row_off, int32_t type)
{
  if (type != vgn::kBoolean) return false;
  const double *b = &h.shape[row_off];
  if (b[vgn::row::BoolOp] == 0.) return true;
  return boolean_has_union(h, row_off + (int32_t)b[vgn::row::BoolLeftRow], (int32_t)b[vgn::row::BoolLeftType]) ||
         boolean_has_union(h, row_off + (int32_t)b[vgn::row::BoolRightRow], (int32_t)b[vgn::row::BoolRightType]);
}

int vgn_shape_batch(const vgn_geometry *gc, int32_t lv, int32_t op, int64_t n, const double *px, const double *py,
                    const double *pz, const double *dx, const double *dy, const double *dz, const double *step_max,
                    double *out, int flags, void *stream)
{
  vgn_geometry *g = const_cast<vgn_geometry *>(gc);
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (lv < 0 || lv >= (int32_t)g->host.lv.size()) return fail(VGN_ERR_ARG, "bad logical volume");
  if (op < VGN_OP_DISTANCE_TO_IN || op > VGN_OP_INSIDE) return fail(VGN_ERR_ARG, "bad shape operation");
  if (op == VGN_OP_INSIDE && boolean_has_union(g->host, g->host.lv[lv].shape_row, g->host.lv[lv].shape))
    return fail(VGN_ERR_UNSUPPORTED, "Inside of a boolean union takes its operands' normals, which are not computed");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n == 0) return VGN_OK;
  const bool needdir = op <= VGN_OP_DISTANCE_TO_OUT;
  if (!px || !py || !pz || !out || (needdir && (!dx || !dy || !dz))) return fail(VGN_ERR_ARG, "null array argument");
  if ((flags & VGN_PRECISION_MIXED) != 0) return fail(VGN_ERR_UNSUPPORTED, "shape queries are FP64 only");
  DeviceGuard guard(g->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int type   = g->host.lv[lv].shape;
  const double *row = g->view.shape + g->host.lv[lv].shape_row;
  const double *smax = needdir ? step_max : nullptr;  // only the distance ops read it
  const int kind     = needdir ? classify({px, py, pz, dx, dy, dz, smax, out}) : classify({px, py, pz, out});
  if (kind < 0) return fail(VGN_ERR_ARG, "mix of host and device pointers");
  if (kind == 1) {
    cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_shape_fp64)(op, type, row, n, px, py, pz, dx, dy, dz, smax,
                                                                     out, max_blocks(g), s);
    return e == cudaSuccess ? VGN_OK : cuda_fail(e, "shape kernel launch");
  }
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  const size_t nd = (size_t)n * sizeof(double);
  void *ws = workspace(g, carve_bytes({nd, nd, nd, nd, nd, nd, nd, nd}));
  if (!ws) return fail(VGN_ERR_NOMEM, "device staging workspace allocation failed");
  Carve c{static_cast<char *>(ws)};
  double *b[7];
  for (int k = 0; k < 7; ++k) b[k] = c.take<double>(n);
  double *dout = c.take<double>(n);
  const double *src[7] = {px, py, pz, dx, dy, dz, smax};
  const int ncopy      = needdir ? 6 : 3;
  cudaError_t e        = cudaSuccess;
  for (int k = 0; k < ncopy && e == cudaSuccess; ++k) e = cudaMemcpyAsync(b[k], src[k], nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && smax) e = cudaMemcpyAsync(b[6], smax, nd, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  e = VGN_KSET_FN(g->host.kset(), launch_shape_fp64)(op, type, row, n, b[0], b[1], b[2], b[3], b[4], b[5],
                                                       smax ? b[6] : nullptr, dout, max_blocks(g), s);
  if (e != cudaSuccess) return cuda_fail(e, "shape kernel launch");
  e = cudaMemcpyAsync(out, dout, nd, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  return check_status(g, s);
}

int vgn_set_step_config(vgn_geometry *g, int flags, int32_t variant, int32_t sort_kbits)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  const int m = (flags & VGN_PRECISION_MIXED) ? 1 : 0;
  if (variant < 0 || variant >= vgn::sections::step_variant_count(m != 0))
    return fail(VGN_ERR_ARG, "unknown launch variant");
  if (sort_kbits < 0 || sort_kbits > 6) return fail(VGN_ERR_ARG, "track-binning granularity must be 0..6");
  g->step_variant[m] = variant;
  g->sort_kbits[m]   = sort_kbits;
  return VGN_OK;
}

int vgn_get_step_variant_count(int flags, int32_t *count)
{
  if (!count) return fail(VGN_ERR_ARG, "null argument");
  *count = vgn::sections::step_variant_count((flags & VGN_PRECISION_MIXED) != 0);
  return VGN_OK;
}

int vgn_get_step_config(const vgn_geometry *g, int flags, int32_t *variant, int32_t *sort_kbits)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  const int m = (flags & VGN_PRECISION_MIXED) ? 1 : 0;
  if (variant) *variant = g->step_variant[m];
  if (sort_kbits) *sort_kbits = g->sort_kbits[m];
  return VGN_OK;
}

int vgn_set_safety_binning(vgn_geometry *g, int flags, int32_t kbits)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (kbits < 0 || kbits > 6) return fail(VGN_ERR_ARG, "safety binning granularity must be 0..6");
  g->safety_kbits[(flags & VGN_PRECISION_MIXED) ? 1 : 0] = kbits;
  return VGN_OK;
}

int vgn_get_safety_binning(const vgn_geometry *g, int flags, int32_t *kbits)
{
  if (!g || !kbits) return fail(VGN_ERR_ARG, "null argument");
  *kbits = g->safety_kbits[(flags & VGN_PRECISION_MIXED) ? 1 : 0];
  return VGN_OK;
}

int vgn_set_staging_chunks(vgn_geometry *g, int32_t chunks)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (chunks < 0 || chunks > 64) return fail(VGN_ERR_ARG, "staging pieces must be 0..64");
  std::lock_guard<std::mutex> lock(g->ws_mutex);
  g->staging_chunks = chunks;
  return VGN_OK;
}

int vgn_get_staging_chunks(const vgn_geometry *g, int32_t *chunks)
{
  if (!g || !chunks) return fail(VGN_ERR_ARG, "null argument");
  *chunks = g->staging_chunks;
  return VGN_OK;
}

int vgn_autotune_step(vgn_geometry *g, int64_t n, const double *px, const double *py, const double *pz,
                      const double *dx, const double *dy, const double *dz, const double *step_limit,
                      const vgn_state *in, vgn_state *out, double *step, double *safety, int flags, void *stream,
                      int32_t *variant, int32_t *sort_kbits, float *best_ms)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n <= 0) return fail(VGN_ERR_ARG, "autotuning needs a non-empty batch");
  DeviceGuard guard(g->device);
  if (classify({px, py, pz, dx, dy, dz, step_limit, in, out, step, safety}) != 1)
    return fail(VGN_ERR_ARG, "autotuning needs device pointers");
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  const int m      = mixed ? 1 : 0;
  cudaStream_t s   = static_cast<cudaStream_t>(stream);
  vgn::StepArgs a{};
  a.n = n; a.px = px; a.py = py; a.pz = pz; a.dx = dx; a.dy = dy; a.dz = dz; a.slimit = step_limit;
  a.in = in; a.out = out; a.step = step; a.safety = safety;
  a.reloc      = (flags & VGN_NO_RELOCATE) ? 0 : 1;
  a.max_blocks = max_blocks(g);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "cudaEventCreate");
  // time one configuration: a warm-up call, then the mean of two
  auto time_cfg = [&](float &ms) -> int {
    int r = enqueue_step(g, a, mixed, s);
    if (r != VGN_OK) return r;
    cudaEventRecord(e0, s);
    for (int k = 0; k < 2 && r == VGN_OK; ++k) r = enqueue_step(g, a, mixed, s);
    cudaEventRecord(e1, s);
    if (r != VGN_OK) return r;
    if (cudaEventSynchronize(e1) != cudaSuccess) return cuda_fail(cudaGetLastError(), "autotune timing");
    cudaEventElapsedTime(&ms, e0, e1);
    ms *= 0.5f;
    return VGN_OK;
  };
  // launch shape and the step's binning, with the safety pass on a 2^6-per-axis position order;
  // then the safety pass's order with the chosen step configuration
  static const int kSort[] = {0, 3, 4, 5, 6};
  static const int kSafetySort[] = {0, 4, 5, 6};
  float best = 3.4e38f;
  int bv = 0, bk = 0, bs = 0, rc = VGN_OK;
  g->safety_kbits[m] = safety ? 6 : 0;
  for (int v = 0; v < vgn::sections::step_variant_count(m != 0) && rc == VGN_OK; ++v) {
    for (int k : kSort) {
      g->step_variant[m] = v;
      g->sort_kbits[m]   = k;
      float ms           = 0.f;
      if ((rc = time_cfg(ms)) != VGN_OK) break;
      if (ms < best) best = ms, bv = v, bk = k;
    }
  }
  g->step_variant[m] = bv;
  g->sort_kbits[m]   = bk;
  bs                 = g->safety_kbits[m];
  if (safety) {
    best = 3.4e38f;
    for (int k : kSafetySort) {
      if (rc != VGN_OK) break;
      g->safety_kbits[m] = k;
      float ms           = 0.f;
      if ((rc = time_cfg(ms)) != VGN_OK) break;
      if (ms < best) best = ms, bs = k;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g->safety_kbits[m] = bs;
  if (rc != VGN_OK) return rc;
  if (variant) *variant = bv;
  if (sort_kbits) *sort_kbits = bk;
  if (best_ms) *best_ms = best;
  return check_status(g, s);
}

int vgn_walk_batch(const vgn_geometry *g, int64_t n, double *px, double *py, double *pz, const double *dx,
                   const double *dy, const double *dz, const double *step_limit, vgn_state *state,
                   int32_t max_steps, int32_t *nsteps, int flags, void *stream)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0 || max_steps < 0) return fail(VGN_ERR_ARG, "negative batch size or step count");
  if (n == 0) return VGN_OK;
  if (!px || !py || !pz || !dx || !dy || !dz || !step_limit || !state || !nsteps)
    return fail(VGN_ERR_ARG, "null array argument");
  DeviceGuard guard(g->device);
  if (classify({px, py, pz, dx, dy, dz, step_limit, state, nsteps}) != 1)
    return fail(VGN_ERR_ARG, "device pointers required");
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  cudaStream_t s   = static_cast<cudaStream_t>(stream);
  // tracks binned like the step's (direction octant, then cell) when the geometry bins its
  // steps; the scratch is stream-ordered (pool_alloc), so walks on several streams of one
  // geometry do not share it
  const int kbits  = g->sort_kbits[mixed ? 1 : 0];
  uint32_t *sort   = nullptr, *perm = nullptr;
  // small batches walk unbinned: the histogram scan over up to 2^21 bins would cost more
  // than the warp coherence it buys
  constexpr int64_t kWalkBinMin = 32768;
  if (kbits > 0 && n >= kWalkBinMin && n <= (int64_t)UINT32_MAX) {
    const size_t words = vgn::bin_scratch_words(n, kbits) + (size_t)n;
    if (pool_alloc(g->device, words * sizeof(uint32_t), s, reinterpret_cast<void **>(&sort)) != cudaSuccess) {
      cudaGetLastError();
      return fail(VGN_ERR_NOMEM, "walk binning scratch allocation failed");
    }
    vgn::BinParams b = g->bin;
    b.kbits          = kbits;
    for (int k = 0; k < 3; ++k) b.scale[k] = g->bin.scale[k] * (float)(1 << kbits);
    perm          = sort + vgn::bin_scratch_words(n, kbits);
    cudaError_t e = vgn::launch_bin_tracks(n, px, py, pz, dx, dy, dz, b, sort, perm, max_blocks(g), s);
    if (e != cudaSuccess) {
      cudaFreeAsync(sort, s);
      return cuda_fail(e, "walk binning launch");
    }
  }
  // the mixed form's block-grouped launch variants walk chunks of tracks per block with
  // block-grouped steps (walk_kernel_grouped)
  const int variant = g->step_variant[mixed ? 1 : 0];
  cudaError_t e = VGN_KSET_FN(g->host.kset(), launch_walk)(g->view, n, px, py, pz, dx, dy, dz, step_limit, state,
                                                             max_steps, nsteps, perm, mixed, variant, max_blocks(g), s);
  if (sort) cudaFreeAsync(sort, s);
  return e == cudaSuccess ? VGN_OK : cuda_fail(e, "walk kernel launch");
}

// ---- batched uneven workloads ------------------------------------------------
struct vgn_batch {
  int device  = 0;
  int num_sms = 0;
  uint32_t *d_queue = nullptr;  // work-queue counter of the persistent launch
  vgn::JobTable jt{};
  std::vector<vgn_step_job> jobs;
  std::vector<vgn::BinParams> bins;
  std::vector<uint32_t *> d_sort;  // per-job binning scratch: keys | histogram | permutation
  std::vector<size_t> sort_words;
  bool mixed    = false;
  int kset = 0;  // the kernel set every job's geometry can run on (0 full_ranges, 1 sections, 2 booleans)
  int safety_kbits = 0;   // the safety pass's own position-only order (0 = the step's)
  int reloc     = 1;
  int variant   = 0;
  int kbits     = 0;
};

namespace {

// (re)build the per-job visit orders for `kbits` (0 = none); allocates only when a job's
// scratch is too small
int batch_configure(vgn_batch *b, int kbits, int ks)
{
  const size_t nj = b->jobs.size();
  b->d_sort.resize(nj, nullptr);
  b->sort_words.resize(nj, 0);
  b->bins.resize(2 * nj);  // per job: the step's order, the safety pass's order
  for (size_t k = 0; k < nj; ++k) {
    vgn::JobRec &r = b->jt.job[k];
    r.perm         = nullptr;
    r.perm_safety  = nullptr;
    const int kss  = r.safety ? ks : 0;
    if ((kbits == 0 && kss == 0) || r.n == 0 || r.n > (int64_t)UINT32_MAX) continue;
    size_t head = kbits > 0 ? vgn::bin_scratch_words(r.n, kbits) : 0;
    if (kss > 0 && vgn::bin_scratch_words(r.n, kss) > head) head = vgn::bin_scratch_words(r.n, kss);
    const size_t need = head + (size_t)r.n * ((kbits > 0 ? 1 : 0) + (kss > 0 ? 1 : 0));
    if (need > b->sort_words[k]) {
      if (b->d_sort[k]) cudaFree(b->d_sort[k]);
      b->d_sort[k]     = nullptr;
      b->sort_words[k] = 0;
      if (cudaMalloc(&b->d_sort[k], need * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        return fail(VGN_ERR_NOMEM, "batch binning scratch allocation failed");
      }
      b->sort_words[k] = need;
    }
    uint32_t *next = b->d_sort[k] + head;
    for (int o = 0; o < 2; ++o) {
      const int kb = o == 0 ? kbits : kss;
      if (kb == 0) continue;
      vgn::BinParams bp = b->jobs[k].geom->bin;
      bp.kbits          = kb;
      bp.octants        = o == 0 ? 1 : 0;
      for (int a = 0; a < 3; ++a) bp.scale[a] = b->jobs[k].geom->bin.scale[a] * (float)(1 << kb);
      b->bins[2 * k + o] = bp;
      (o == 0 ? r.perm : r.perm_safety) = next;
      next += r.n;
    }
  }
  b->kbits        = kbits;
  b->safety_kbits = ks;
  return VGN_OK;
}

int batch_enqueue(vgn_batch *b, cudaStream_t s)
{
  for (int k = 0; k < b->jt.n_jobs; ++k) {
    const vgn::JobRec &r = b->jt.job[k];
    const uint32_t *orders[2] = {r.perm, r.perm_safety};
    for (int o = 0; o < 2; ++o) {
      if (!orders[o]) continue;
      cudaError_t e = vgn::launch_bin_tracks(r.n, r.px, r.py, r.pz, r.dx, r.dy, r.dz, b->bins[2 * k + o],
                                             b->d_sort[k], const_cast<uint32_t *>(orders[o]), b->num_sms * 32, s);
      if (e != cudaSuccess) return cuda_fail(e, "batch track binning launch");
    }
  }
  cudaError_t e = VGN_KSET_FN(b->kset, launch_multi_step)(b->jt, b->d_queue, b->mixed, b->reloc, b->num_sms, b->variant, s);
  return e == cudaSuccess ? VGN_OK : cuda_fail(e, "batch step launch");
}

}  // namespace

int vgn_batch_create(int device, vgn_batch **out)
{
  if (!out) return fail(VGN_ERR_ARG, "null output pointer");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return fail(VGN_ERR_ARG, "no such CUDA device");
  }
  vgn_batch *b = new (std::nothrow) vgn_batch();
  if (!b) return fail(VGN_ERR_NOMEM, "host allocation failed");
  b->device = device;
  DeviceGuard guard(device);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&b->d_queue, 256) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return fail(VGN_ERR_NOMEM, "batch work-queue allocation failed");
  }
  *out = b;
  return VGN_OK;
}

int vgn_batch_free(vgn_batch *b)
{
  if (!b) return VGN_OK;
  DeviceGuard guard(b->device);
  for (uint32_t *p : b->d_sort)
    if (p) cudaFree(p);
  if (b->d_queue) cudaFree(b->d_queue);
  delete b;
  return VGN_OK;
}

int vgn_batch_set_jobs(vgn_batch *b, int n_jobs, const vgn_step_job *jobs, int flags, int32_t variant,
                       int32_t sort_kbits)
{
  if (!b) return fail(VGN_ERR_ARG, "null batch");
  if (n_jobs < 1 || n_jobs > VGN_BATCH_MAX_JOBS || !jobs)
    return fail(VGN_ERR_ARG, "a batch holds 1.." + std::to_string(VGN_BATCH_MAX_JOBS) + " jobs");
  if (variant < 0 || variant >= vgn::sections::multi_variant_count()) return fail(VGN_ERR_ARG, "unknown launch variant");
  if (sort_kbits < 0 || sort_kbits > 6) return fail(VGN_ERR_ARG, "track-binning granularity must be 0..6");
  DeviceGuard guard(b->device);
  uint64_t chunks = 0;
  for (int k = 0; k < n_jobs; ++k) {
    const vgn_step_job &j = jobs[k];
    if (!j.geom || j.geom->device != b->device)
      return fail(VGN_ERR_ARG, "job " + std::to_string(k) + ": geometry missing or on another device");
    if (j.n < 0) return fail(VGN_ERR_ARG, "job " + std::to_string(k) + ": negative batch size");
    if (j.n > 0) {
      if (!j.px || !j.py || !j.pz || !j.dx || !j.dy || !j.dz || !j.step_limit || !j.in || !j.out || !j.step)
        return fail(VGN_ERR_ARG, "job " + std::to_string(k) + ": null array argument");
      if (classify({j.px, j.py, j.pz, j.dx, j.dy, j.dz, j.step_limit, j.in, j.out, j.step, j.safety}) != 1)
        return fail(VGN_ERR_ARG, "job " + std::to_string(k) + ": device pointers required");
    }
    chunks += ((uint64_t)j.n + 31) / 32;
  }
  if (chunks >= UINT32_MAX) return fail(VGN_ERR_ARG, "too many tracks in one batch");
  b->jobs.assign(jobs, jobs + n_jobs);
  b->jt        = vgn::JobTable{};
  b->jt.n_jobs = n_jobs;
  uint32_t c   = 0;
  for (int k = 0; k < n_jobs; ++k) {
    const vgn_step_job &j = jobs[k];
    vgn::JobRec &r        = b->jt.job[k];
    r.g = j.geom->view;
    r.px = j.px; r.py = j.py; r.pz = j.pz; r.dx = j.dx; r.dy = j.dy; r.dz = j.dz; r.slimit = j.step_limit;
    r.in = j.in; r.out = j.out; r.step = j.step; r.safety = j.safety;
    r.n                   = j.n;
    r.perm                = nullptr;
    r.perm_safety         = nullptr;
    b->jt.chunk_begin[k]  = c;
    c += (uint32_t)(((uint64_t)j.n + 31) / 32);
  }
  b->jt.chunk_begin[n_jobs] = c;
  b->kset                   = 0;
  for (int k = 0; k < n_jobs; ++k) b->kset = std::max(b->kset, jobs[k].geom->host.kset());
  b->mixed                  = (flags & VGN_PRECISION_MIXED) != 0;
  b->reloc                  = (flags & VGN_NO_RELOCATE) ? 0 : 1;
  b->variant                = variant;
  return batch_configure(b, sort_kbits, b->safety_kbits);
}

int vgn_batch_step(vgn_batch *b, void *stream)
{
  if (!b) return fail(VGN_ERR_ARG, "null batch");
  if (b->jt.n_jobs == 0) return fail(VGN_ERR_ARG, "batch has no jobs");
  DeviceGuard guard(b->device);
  return batch_enqueue(b, static_cast<cudaStream_t>(stream));
}

int vgn_batch_synchronize(vgn_batch *b, void *stream)
{
  if (!b) return fail(VGN_ERR_ARG, "null batch");
  DeviceGuard guard(b->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc         = VGN_OK;
  for (const vgn_step_job &j : b->jobs) {
    const int r = check_status(j.geom, s);
    if (r != VGN_OK && rc == VGN_OK) rc = r;
  }
  if (b->jobs.empty()) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
  }
  return rc;
}

int vgn_batch_autotune(vgn_batch *b, void *stream, int32_t *variant, int32_t *sort_kbits, float *best_ms)
{
  if (!b) return fail(VGN_ERR_ARG, "null batch");
  if (b->jt.n_jobs == 0) return fail(VGN_ERR_ARG, "batch has no jobs");
  DeviceGuard guard(b->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "cudaEventCreate");
  // launch shape and the step's binning with the safety pass on a 2^6-per-axis position order,
  // then the safety pass's order with that configuration
  static const int kSort[] = {0, 3, 4, 5, 6};
  static const int kSafetySort[] = {0, 4, 5, 6};
  bool any_safety = false;
  for (int k = 0; k < b->jt.n_jobs; ++k) any_safety = any_safety || b->jt.job[k].safety;
  float best = 3.4e38f;
  int bv = 0, bk = 0, bs = any_safety ? 6 : 0, rc = VGN_OK;
  for (int k : kSort) {
    if ((rc = batch_configure(b, k, bs)) != VGN_OK) break;
    for (int v = 0; v < vgn::sections::multi_variant_count() && rc == VGN_OK; ++v) {
      b->variant = v;
      if ((rc = batch_enqueue(b, s)) != VGN_OK) break;  // warm-up
      cudaEventRecord(e0, s);
      for (int r = 0; r < 2 && rc == VGN_OK; ++r) rc = batch_enqueue(b, s);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "batch autotune timing");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms *= 0.5f;
      if (ms < best) best = ms, bv = v, bk = k;
    }
    if (rc != VGN_OK) break;
  }
  b->variant = bv;
  if (any_safety && rc == VGN_OK) {
    float best_s = 3.4e38f;
    int bss      = bs;
    for (int ks : kSafetySort) {
      if ((rc = batch_configure(b, bk, ks)) != VGN_OK) break;
      if ((rc = batch_enqueue(b, s)) != VGN_OK) break;  // warm-up
      cudaEventRecord(e0, s);
      for (int r = 0; r < 2 && rc == VGN_OK; ++r) rc = batch_enqueue(b, s);
      cudaEventRecord(e1, s);
      if (rc != VGN_OK) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "batch autotune timing");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms *= 0.5f;
      if (ms < best_s) best_s = ms, bss = ks;
    }
    bs   = bss;
    best = best_s;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int rc2 = batch_configure(b, bk, bs);
  if (rc != VGN_OK) return rc;
  if (rc2 != VGN_OK) return rc2;
  if (variant) *variant = bv;
  if (sort_kbits) *sort_kbits = bk;
  if (best_ms) *best_ms = best;
  return vgn_batch_synchronize(b, stream);
}

// Binned step whose binning scratch is the library's static device buffer
// (kernels_sort.cu): no cudaMalloc, no cudaFree, no staging workspace.
int vgn_compute_step_batch_static(const vgn_geometry *g, int64_t n, const double *px, const double *py,
                                  const double *pz, const double *dx, const double *dy, const double *dz,
                                  const double *step_limit, const vgn_state *in, vgn_state *out, double *step,
                                  double *safety, int flags, int32_t sort_kbits, void *stream)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  if (n < 0) return fail(VGN_ERR_ARG, "negative batch size");
  if (n > VGN_STATIC_SCRATCH_MAX_TRACKS)
    return fail(VGN_ERR_ARG, "batch of " + std::to_string(n) + " tracks exceeds the static binning scratch (at most " +
                                 std::to_string(VGN_STATIC_SCRATCH_MAX_TRACKS) + " tracks per call)");
  if (sort_kbits < 1 || sort_kbits > VGN_STATIC_SCRATCH_MAX_KBITS)
    return fail(VGN_ERR_ARG, "sort_kbits must be 1.." + std::to_string(VGN_STATIC_SCRATCH_MAX_KBITS));
  if (n == 0) return VGN_OK;
  if (!px || !py || !pz || !dx || !dy || !dz || !step_limit || !in || !out || !step)
    return fail(VGN_ERR_ARG, "null array argument");
  DeviceGuard guard(g->device);
  if (classify({px, py, pz, dx, dy, dz, step_limit, in, out, step, safety}) != 1)
    return fail(VGN_ERR_ARG, "device pointers required: this entry point stages no host buffers");
  uint32_t *scratch = nullptr;
  cudaError_t e     = vgn::static_scratch(&scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static binning scratch)");
  const bool mixed = (flags & VGN_PRECISION_MIXED) != 0;
  cudaStream_t s   = static_cast<cudaStream_t>(stream);
  vgn::BinParams b = g->bin;
  b.kbits          = sort_kbits;
  for (int k = 0; k < 3; ++k) b.scale[k] = g->bin.scale[k] * (float)(1 << sort_kbits);
  // keys [n] | histogram [8 * 2^(3k)], zeroed by launch_bin_tracks | tile sums | permutation [n]
  uint32_t *perm = scratch + (size_t)n + ((size_t)8 << (3 * sort_kbits)) + vgn::kScanSumWords;
  e = vgn::launch_bin_tracks(n, px, py, pz, dx, dy, dz, b, scratch, perm, max_blocks(g), s);
  if (e != cudaSuccess) return cuda_fail(e, "track binning launch");
  vgn::StepArgs a{};
  a.n = n; a.px = px; a.py = py; a.pz = pz; a.dx = dx; a.dy = dy; a.dz = dz; a.slimit = step_limit;
  a.in = in; a.out = out; a.step = step; a.safety = safety;
  a.reloc      = (flags & VGN_NO_RELOCATE) ? 0 : 1;
  a.max_blocks = max_blocks(g);
  a.perm       = perm;
  e = VGN_KSET_FN(g->host.kset(), launch_step)(g->view, a, mixed, g->step_variant[mixed ? 1 : 0], s);
  return e == cudaSuccess ? VGN_OK : cuda_fail(e, "step kernel launch");
}

int vgn_set_device_limits(vgn_geometry *g, int32_t stack_entries, int32_t levels)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (stack_entries < 2 || stack_entries > vgn::kStackSize || levels < 1 || levels > vgn::kMaxLevels)
    return fail(VGN_ERR_ARG, "device limits out of range (stack 2..32, levels 1..30)");
  g->view.stack_limit = stack_entries;
  g->view.level_limit = levels;
  return VGN_OK;
}

int vgn_synchronize(const vgn_geometry *g, void *stream)
{
  if (!g) return fail(VGN_ERR_ARG, "null geometry");
  if (g->device == VGN_HOST_ONLY) return fail(VGN_ERR_ARG, "geometry was closed on the host only");
  DeviceGuard guard(g->device);
  return check_status(g, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
