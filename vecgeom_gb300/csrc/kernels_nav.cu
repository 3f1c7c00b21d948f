// kernels_nav.cu -- navigation kernels: step, safety, locate and shape queries,
// each in an all-FP64 form and (step, safety, locate) a mixed-precision form.
//
// Compiled with -fmad=false: every FP64 expression keeps the reference's
// operation order (no contraction into FMA), so results are bit-identical to
// the reference's scalar CPU navigator.  The FP32 interval code of the mixed
// form uses explicitly rounded intrinsics, which are never contracted.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/vgnav.h"
#include "launch.h"
#include "nav_step.cuh"

namespace vgn {
namespace dev {
inline namespace VGN_KSET {

__device__ __forceinline__ State load_state(const vgn_state *s, int64_t i)
{
  const uint32_t *w = reinterpret_cast<const uint32_t *>(s + i);
  State r;
  r.nav_ind     = __ldg(w);
  r.last_exited = __ldg(w + 1);
  r.on_boundary = __ldg(w + 2) & 0xffu;
  return r;
}

__device__ __forceinline__ void store_state(vgn_state *s, int64_t i, const State &st)
{
  uint32_t *w = reinterpret_cast<uint32_t *>(s + i);
  w[0]        = st.nav_ind;
  w[1]        = st.last_exited;
  w[2]        = st.on_boundary & 0xffu;
}

template <bool MIXED, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) step_kernel(GeomView g, int64_t n, const double *__restrict__ px,
                                                   const double *__restrict__ py, const double *__restrict__ pz,
                                                   const double *__restrict__ dx, const double *__restrict__ dy,
                                                   const double *__restrict__ dz, const double *__restrict__ slimit,
                                                   const vgn_state *__restrict__ in, vgn_state *__restrict__ out,
                                                   double *__restrict__ step, int reloc,
                                                   const uint32_t *__restrict__ perm)
{
  // the step only: safeties come from safety_kernel, a separate pass over the same order
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)__ldg(perm + t) : t;  // binned visit order, results stay at index i
    const State s   = load_state(in, i);
    State o       = s;
    double st;
    if (!ni_valid(g, s.nav_ind) || (s.last_exited != 0 && !ni_valid(g, s.last_exited))) {
      raise_error(g, kErrState);
      st = 0.;
    } else {
      st = nav_step<MIXED>(g, d3(px[i], py[i], pz[i]), d3(dx[i], dy[i], dz[i]), slimit[i], s, o, reloc != 0);
    }
    step[i] = st;
    store_state(out, i, o);
  }
}

// Step kernel of the mixed form with the FP64 DistanceToIn of the BVH candidates grouped by
// shape type across the whole block.  Per round of BLOCK tracks:
//   1. each thread: step start, FP32 traversal into its candidate queue, its local point and
//      direction into shared memory, and for every candidate that may be computed ahead
//      (step_pending) a place in its shape type's part of the block's item list;
//   2. the list is laid out type after type, each part padded to a multiple of 32 entries;
//   3. every warp takes 32 consecutive entries at a time -- candidates of one shape type,
//      from any thread of the block -- and computes their DistanceToIn into the owners' slots;
//   4. each thread: the reference's acceptance rule over its queue in visit order
//      (step_replay), then PrepareOutState and relocation.
// Every value is computed by the same FP64 code as in the other kernels, and a candidate's
// DistanceToIn does not depend on when or by which thread it is computed, so the results
// are those of step_kernel.  Shared memory after the per-thread words: local points and
// directions (6 doubles per thread), per-type counters and offsets, the item list (16-bit
// entries: owner thread << 4 | queue slot; 0xffff pads).
#if VGN_SMEM_STACK
constexpr int kGroupPad        = 32;
constexpr uint16_t kGroupEmpty = 0xffffu;
static_assert(kMaxStepCand <= 16, "queue slot in 4 bits of an item entry");
template <int BLOCK>
struct GroupLayout {
  static_assert(BLOCK <= 1024 && BLOCK % 32 == 0, "owner thread in 12 bits; whole warps");
  static constexpr int kListCap       = BLOCK * kMaxStepCand + kNumShapes * kGroupPad;
  static constexpr size_t kThreadBytes = (size_t)kStepSmemWords * BLOCK * sizeof(uint32_t);
  static constexpr size_t kRayBytes    = (size_t)6 * BLOCK * sizeof(double);
  static constexpr size_t kCountBytes  = 64 * sizeof(uint32_t);  // counters [16], offsets [17], chunk counter at 48
  static constexpr size_t kBytes       = kThreadBytes + kRayBytes + kCountBytes + (size_t)kListCap * sizeof(uint16_t);
};

// One navigation step (nav_step<true> semantics) of every live thread of the block, with the
// candidates' DistanceToIn grouped by shape type across the block.  Called by every thread of
// the block (it holds barriers); `live` threads step from (gp, gd, s) and receive the step in
// `st` and the propagated state in `o`.
template <int BLOCK>
__device__ __forceinline__ void grouped_step(const GeomView &g, bool live, D3 gp, D3 gd, double slimit,
                                             const State &s, State &o, bool reloc, double &st)
{
  using L       = GroupLayout<BLOCK>;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double *ray   = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(vgn_step_smem) + L::kThreadBytes);
  uint32_t *cnt = reinterpret_cast<uint32_t *>(ray + 6 * BLOCK);
  uint32_t *off = cnt + 16;  // off[t]: first entry of type t; off[kNumShapes]: list length
  uint16_t *list = reinterpret_cast<uint16_t *>(cnt + 64);
  const int *cand_pv = reinterpret_cast<const int *>(vgn_step_smem + kStackSize * BLOCK);
  const SlotWords own{vgn_step_smem + tid, BLOCK};
  // 1. step start and traversal (the counters were cleared by the previous round or at entry)
  D3 lp = d3(0., 0., 0.), ld = d3(0., 0., 0.);
  LVRec lv{};
  int hit = -1, last = 0;
  MixedRay r;
  StepCands c;
  c.n = 0;
  FI stepI{0.f, 0.f};
  unsigned done = 0;
  st = 0.;
  if (live) {
    step_begin(g, gp, gd, slimit, s, lp, ld, lv, st);
    make_ray(r, lp, ld);
    stepI = fi(st);
    last  = ni_top(g, s.last_exited);
    if (lv.nd > 0) {
      bvh_collect_step_mixed(g, lv, r, st, stepI, last, hit, c);
      unsigned present;
      done = step_pending(c, stepI, present);
      ray[tid]             = lp.x;
      ray[BLOCK + tid]     = lp.y;
      ray[2 * BLOCK + tid] = lp.z;
      ray[3 * BLOCK + tid] = ld.x;
      ray[4 * BLOCK + tid] = ld.y;
      ray[5 * BLOCK + tid] = ld.z;
      for (unsigned rest = done; rest; rest &= rest - 1) {
        const int q  = __ffs(rest) - 1;
        own.word(q) = atomicAdd(&cnt[c.type(q)], 1u);  // place within its type
      }
    }
  }
  __syncthreads();
  // 2. list layout: exclusive scan of the padded per-type counts, pads marked empty
  if (warp == 0) {
    const uint32_t v      = lane < kNumShapes ? cnt[lane] : 0u;
    const uint32_t padded = (v + kGroupPad - 1) & ~(uint32_t)(kGroupPad - 1);
    uint32_t incl         = padded;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    const uint32_t excl = incl - padded;
    if (lane <= kNumShapes) off[lane] = excl;
    for (int u = 0; u < kNumShapes; ++u) {
      const uint32_t cu = __shfl_sync(0xffffffffu, v, u);
      const uint32_t ou = __shfl_sync(0xffffffffu, excl, u);
      const uint32_t pu = __shfl_sync(0xffffffffu, padded, u);
      if (cu + (uint32_t)lane < pu) list[ou + cu + lane] = kGroupEmpty;
    }
  }
  __syncthreads();
  for (unsigned rest = done; rest; rest &= rest - 1) {
    const int q = __ffs(rest) - 1;
    list[off[c.type(q)] + own.word(q)] = (uint16_t)((tid << 4) | q);
  }
  __syncthreads();
  // 3. 32 entries of one shape type per warp and turn
  const uint32_t total = off[kNumShapes];
  for (uint32_t j = (uint32_t)warp * 32u; j < total; j += BLOCK) {
    const uint16_t e = list[j + lane];
    if (e != kGroupEmpty) {
      const int ow = e >> 4, q = e & 15;
      const D3 olp = d3(ray[ow], ray[BLOCK + ow], ray[2 * BLOCK + ow]);
      const D3 old = d3(ray[3 * BLOCK + ow], ray[4 * BLOCK + ow], ray[5 * BLOCK + ow]);
      SlotWords{vgn_step_smem + ow, BLOCK}.put(q, pv_dist_in(g, cand_pv[q * BLOCK + ow], olp, old, kInfLength));
    }
  }
  if (tid < 16) cnt[tid] = 0;  // for the next round; no thread reads the counters until then
  __syncthreads();
  // 4. acceptance in visit order, out state, relocation
  if (live) {
    if (lv.nd > 0) step_replay(g, r, c, done, own, st, stepI, last, hit);
    st = step_finish<true>(g, lp, ld, slimit, s, o, reloc, st, hit);
  }
}

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) step_kernel_grouped(GeomView g, int64_t n, const double *__restrict__ px,
                                                           const double *__restrict__ py, const double *__restrict__ pz,
                                                           const double *__restrict__ dx, const double *__restrict__ dy,
                                                           const double *__restrict__ dz, const double *__restrict__ slimit,
                                                           const vgn_state *__restrict__ in, vgn_state *__restrict__ out,
                                                           double *__restrict__ step, int reloc,
                                                           const uint32_t *__restrict__ perm)
{
  uint32_t *cnt = reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(vgn_step_smem) +
                                               GroupLayout<BLOCK>::kThreadBytes + GroupLayout<BLOCK>::kRayBytes);
  if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t base = (int64_t)blockIdx.x * BLOCK; base < n; base += (int64_t)gridDim.x * BLOCK) {
    const int64_t t = base + threadIdx.x;
    int64_t i       = 0;
    State s{}, o{};
    bool ok = false;
    D3 gp = d3(0., 0., 0.), gd = d3(0., 0., 0.);
    double sl = 0.;
    if (t < n) {
      i  = perm ? (int64_t)__ldg(perm + t) : t;
      s  = load_state(in, i);
      o  = s;
      ok = ni_valid(g, s.nav_ind) && !(s.last_exited != 0 && !ni_valid(g, s.last_exited));
      if (!ok) raise_error(g, kErrState);
      if (ok) {
        gp = d3(px[i], py[i], pz[i]);
        gd = d3(dx[i], dy[i], dz[i]);
        sl = slimit[i];
      }
    }
    double st;
    grouped_step<BLOCK>(g, ok, gp, gd, sl, s, o, reloc != 0, st);
    if (t < n) {
      step[i] = ok ? st : 0.;
      store_state(out, i, o);
    }
  }
}

// Transport loop (walk_kernel semantics) with block-grouped steps.  Each block walks its own
// chunk of kWalkChunk * BLOCK consecutive tracks (of the visit order): a thread whose track has
// left the world (or used max_steps) takes the chunk's next track from a shared-memory counter,
// so the block's threads stay busy until the chunk is done, and every round is one
// grouped_step over the block's live tracks.  A block lives as long as its chunk, so work of
// higher-priority streams finds free multiprocessors within about that time.
constexpr int kWalkChunk = 4;

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) walk_kernel_grouped(GeomView g, int64_t n, double *__restrict__ px,
                                                           double *__restrict__ py, double *__restrict__ pz,
                                                           const double *__restrict__ dx, const double *__restrict__ dy,
                                                           const double *__restrict__ dz,
                                                           const double *__restrict__ slimit,
                                                           vgn_state *__restrict__ state, int max_steps,
                                                           int32_t *__restrict__ nsteps,
                                                           const uint32_t *__restrict__ perm)
{
  uint32_t *cnt  = reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(vgn_step_smem) +
                                                GroupLayout<BLOCK>::kThreadBytes + GroupLayout<BLOCK>::kRayBytes);
  uint32_t *next = cnt + 48;  // the chunk's track counter (after the counters and offsets)
  for (int64_t base = (int64_t)blockIdx.x * kWalkChunk * BLOCK; base < n;
       base += (int64_t)gridDim.x * kWalkChunk * BLOCK) {
    const int64_t chunk_n = n - base < (int64_t)kWalkChunk * BLOCK ? n - base : (int64_t)kWalkChunk * BLOCK;
    if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) *next = 0;
    __syncthreads();
    int64_t i = -1;  // the thread's track, -1: none
    bool more = true;  // the chunk may still hold tracks
    D3 p = d3(0., 0., 0.), d = d3(0., 0., 0.);
    double sl = 0.;
    State s{};
    int k = 0;
    for (;;) {
      while (i < 0 && more) {  // take the chunk's next track that needs a step
        const uint32_t c = atomicAdd(next, 1u);
        if ((int64_t)c >= chunk_n) {
          more = false;
          break;
        }
        const int64_t t = base + c;
        i = perm ? (int64_t)__ldg(perm + t) : t;
        s = load_state(state, i);
        if (s.nav_ind != 0 && (!ni_valid(g, s.nav_ind) || (s.last_exited != 0 && !ni_valid(g, s.last_exited)))) {
          raise_error(g, kErrState);
          nsteps[i] = -1;
          i         = -1;
          continue;
        }
        if (s.nav_ind == 0 || max_steps <= 0) {  // nothing to do: outside the world already
          nsteps[i] = 0;
          i         = -1;
          continue;
        }
        p  = d3(px[i], py[i], pz[i]);
        d  = d3(dx[i], dy[i], dz[i]);
        sl = slimit[i];
        k  = 0;
      }
      const bool live = i >= 0;
      if (!__syncthreads_or(live)) break;
      State o = s;
      double st;
      grouped_step<BLOCK>(g, live, p, d, sl, s, o, true, st);
      if (live) {
        p = d3(p.x + st * d.x, p.y + st * d.y, p.z + st * d.z);
        s = o;
        ++k;
        if (s.nav_ind == 0 || k >= max_steps) {
          px[i] = p.x;
          py[i] = p.y;
          pz[i] = p.z;
          store_state(state, i, s);
          nsteps[i] = k;
          i         = -1;
        }
      }
    }
  }
}
#endif  // VGN_SMEM_STACK

// Persistent multi-job step: every warp repeatedly takes the next 32-track chunk from the
// work queue, finds its job (jobs are laid out back to back in chunk space) and steps
// those tracks in the job's geometry.  The job table is a __grid_constant__ parameter,
// read through the constant path with a warp-uniform index.
template <bool MIXED, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) multi_step_kernel(const __grid_constant__ JobTable jt,
                                                                 uint32_t *__restrict__ queue, int reloc)
{
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t chunk = 0;
    if (lane == 0) chunk = atomicAdd(queue, 1u);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= jt.chunk_begin[jt.n_jobs]) return;
    int lo = 0, hi = jt.n_jobs - 1;  // last job whose first chunk is <= chunk
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jt.chunk_begin[mid] <= chunk) lo = mid;
      else hi = mid - 1;
    }
    const JobRec &j = jt.job[lo];
    const int64_t t = (int64_t)(chunk - jt.chunk_begin[lo]) * 32 + lane;
    if (t < j.n) {  // the job's last chunk may be partly empty
      const int64_t i = j.perm ? (int64_t)__ldg(j.perm + t) : t;
      const State s   = load_state(j.in, i);
      State o         = s;
      double st;
      if (!ni_valid(j.g, s.nav_ind) || (s.last_exited != 0 && !ni_valid(j.g, s.last_exited))) {
        raise_error(j.g, kErrState);
        st = 0.;
      } else {  // safeties come from multi_safety_kernel, launched before this kernel
        st = nav_step<MIXED>(j.g, d3(j.px[i], j.py[i], j.pz[i]), d3(j.dx[i], j.dy[i], j.dz[i]), j.slimit[i], s,
                             o, reloc != 0);
      }
      j.step[i] = st;
      store_state(j.out, i, o);
    }
    __syncwarp();
  }
}

// Transport loop per track: ComputeStepAndPropagatedState, then p += step * d, until the
// track leaves the world (state 0) or after max_steps steps; positions and states are
// updated in place (the loop of TestVGDMLNavigation.cpp:86-102, kept on the device).
template <bool MIXED>
__global__ void __launch_bounds__(128, 6) walk_kernel(GeomView g, int64_t n, double *__restrict__ px,
                                                      double *__restrict__ py, double *__restrict__ pz,
                                                      const double *__restrict__ dx, const double *__restrict__ dy,
                                                      const double *__restrict__ dz,
                                                      const double *__restrict__ slimit, vgn_state *__restrict__ state,
                                                      int max_steps, int32_t *__restrict__ nsteps,
                                                      const uint32_t *__restrict__ perm)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)__ldg(perm + t) : t;  // binned visit order, results stay at index i
    State s         = load_state(state, i);
    if (s.nav_ind != 0 && (!ni_valid(g, s.nav_ind) || (s.last_exited != 0 && !ni_valid(g, s.last_exited)))) {
      raise_error(g, kErrState);
      nsteps[i] = -1;
      continue;
    }
    D3 p            = d3(px[i], py[i], pz[i]);
    const D3 d      = d3(dx[i], dy[i], dz[i]);
    const double sl = slimit[i];
    int k           = 0;
    while (s.nav_ind != 0 && k < max_steps) {
      State o = s;
      const double st = nav_step<MIXED>(g, p, d, sl, s, o, true);
      p               = d3(p.x + st * d.x, p.y + st * d.y, p.z + st * d.z);
      s               = o;
      ++k;
    }
    px[i] = p.x;
    py[i] = p.y;
    pz[i] = p.z;
    store_state(state, i, s);
    nsteps[i] = k;
  }
}

// Safety kernels: 128-thread blocks, each thread's traversal stack and pending daughters in
// dynamic shared memory (bvh_safety_mixed), 28 KiB per block.
#ifndef VGN_SAFETY_MINB
#define VGN_SAFETY_MINB 6  // resident safety blocks per SM the register cap is set for
#endif
constexpr int kSafetyBlock         = 128;
constexpr size_t kSafetySmemBytes = (size_t)kSafetySmemWords * kSafetyBlock * sizeof(uint32_t);

// Safety of one track at its state's volume: VSafetyEstimatorHelper::ComputeSafety
// (VSafetyEstimator.h:98-107), also the safety part of ComputeStepAndSafetyAndPropagatedState
// (VNavigator.h:1014-1064), which takes it at the input state before the step.  With
// `step_checks` the track is rejected like the step kernel rejects it (invalid last-exited
// state too), so a step followed by this pass writes what one fused step would.
__device__ __forceinline__ bool safety_state_ok(const GeomView &g, const State &s, bool step_checks)
{
  return ni_valid(g, s.nav_ind) && !(step_checks && s.last_exited != 0 && !ni_valid(g, s.last_exited));
}

template <bool MIXED>
__device__ __forceinline__ double track_safety(const GeomView &g, const State &s, D3 gp)
{
  Xf m;
  top_matrix(g, s.nav_ind, m);
  const LVRec lv = load_lv(g, pv_lv(g, ni_top(g, s.nav_ind)));
  return safety_local<MIXED>(g, lv, xf_point(m.t, m.r, gp), d3(1., 0., 0.));
}

template <bool MIXED>
__global__ void __launch_bounds__(kSafetyBlock, VGN_SAFETY_MINB) safety_kernel(GeomView g, int64_t n, const double *__restrict__ px,
                                                     const double *__restrict__ py, const double *__restrict__ pz,
                                                     const vgn_state *__restrict__ in, double *__restrict__ safety,
                                                     const uint32_t *__restrict__ perm, int step_checks)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)__ldg(perm + t) : t;
    const State s   = load_state(in, i);
    if (!safety_state_ok(g, s, step_checks != 0)) {
      raise_error(g, kErrState);
      safety[i] = 0.;
      continue;
    }
    safety[i] = track_safety<MIXED>(g, s, d3(px[i], py[i], pz[i]));
  }
}

// Persistent multi-job safety pass over the same job table and chunk space as
// multi_step_kernel, for the jobs that asked for safeties.
template <bool MIXED>
__global__ void __launch_bounds__(kSafetyBlock, VGN_SAFETY_MINB) multi_safety_kernel(const __grid_constant__ JobTable jt,
                                                              uint32_t *__restrict__ queue)
{
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t chunk = 0;
    if (lane == 0) chunk = atomicAdd(queue, 1u);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= jt.chunk_begin[jt.n_jobs]) return;
    int lo = 0, hi = jt.n_jobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jt.chunk_begin[mid] <= chunk) lo = mid;
      else hi = mid - 1;
    }
    const JobRec &j = jt.job[lo];
    const int64_t t = (int64_t)(chunk - jt.chunk_begin[lo]) * 32 + lane;
    if (j.safety && t < j.n) {
      const uint32_t *order = j.perm_safety ? j.perm_safety : j.perm;
      const int64_t i       = order ? (int64_t)__ldg(order + t) : t;
      const State s   = load_state(j.in, i);
      if (!safety_state_ok(j.g, s, true)) {
        raise_error(j.g, kErrState);
        j.safety[i] = 0.;
      } else {
        j.safety[i] = track_safety<MIXED>(j.g, s, d3(j.px[i], j.py[i], j.pz[i]));
      }
    }
    __syncwarp();
  }
}

// GlobalLocator::LocateGlobalPoint(world, p, state, true)
template <bool MIXED>
__global__ void __launch_bounds__(256) locate_kernel(GeomView g, int64_t n, const double *__restrict__ px,
                                                     const double *__restrict__ py, const double *__restrict__ pz,
                                                     vgn_state *__restrict__ out)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    State s{0u, 0u, 0u};
    locate_global_point<MIXED>(g, g.world_pv, d3(px[i], py[i], pz[i]), s.nav_ind, true);
    store_state(out, i, s);
  }
}

// BVH::ApproachNextDaughter (BVH.cpp:395-449) per track over the BVH of logical volume lvs[i];
// a volume id out of range or without daughters, or a last-exited id out of range, is recorded
// as an invalid input (kErrState) and leaves the track's step as it was
__global__ void __launch_bounds__(256) approach_kernel(GeomView g, int64_t n, const int32_t *__restrict__ lvs,
                                                       const double *__restrict__ px, const double *__restrict__ py,
                                                       const double *__restrict__ pz, const double *__restrict__ dx,
                                                       const double *__restrict__ dy, const double *__restrict__ dz,
                                                       const int32_t *__restrict__ last, double *__restrict__ step)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int l      = __ldg(lvs + i);
    const int lastpv = last ? __ldg(last + i) : -1;
    if (l < 0 || l >= g.n_lv || lastpv < -1 || lastpv >= g.n_pv) {
      raise_error(g, kErrState);
      continue;
    }
    const LVRec lv = load_lv(g, l);
    if (lv.nd == 0) {
      raise_error(g, kErrState);
      continue;
    }
    double st = step[i];
    bvh_approach(g, lv, d3(px[i], py[i], pz[i]), d3(dx[i], dy[i], dz[i]), st, lastpv);
    step[i] = st;
  }
}

// unplaced shape queries on one logical volume
template <int OP>
__global__ void __launch_bounds__(256) shape_kernel_fp64(int type, const double *__restrict__ row, int64_t n,
                                                         const double *__restrict__ px, const double *__restrict__ py,
                                                         const double *__restrict__ pz, const double *__restrict__ dx,
                                                         const double *__restrict__ dy, const double *__restrict__ dz,
                                                         const double *__restrict__ step_max, double *__restrict__ out)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const D3 p = d3(px[i], py[i], pz[i]);
    double r;
    if (OP == VGN_OP_DISTANCE_TO_IN)
      r = shape_dist_in(type, row, p, d3(dx[i], dy[i], dz[i]), step_max ? step_max[i] : kInfLength);
    else if (OP == VGN_OP_DISTANCE_TO_OUT)
      r = shape_dist_out(type, row, p, d3(dx[i], dy[i], dz[i]), step_max ? step_max[i] : kInfLength);
    else if (OP == VGN_OP_SAFETY_TO_IN)
      r = shape_safe_in(type, row, p);
    else if (OP == VGN_OP_SAFETY_TO_OUT)
      r = shape_safe_out(type, row, p);
    else if (OP == VGN_OP_CONTAINS)
      r = shape_contains(type, row, p) ? 1. : 0.;
    else
      r = (double)shape_inside(type, row, p);
    out[i] = r;
  }
}

}  // namespace VGN_KSET
}  // namespace dev

namespace VGN_KSET {

// dynamic shared memory of the step-path kernels (traversal stacks and candidate queues)
static constexpr size_t step_smem_bytes(int block) { return (size_t)dev::kStepSmemWords * block * sizeof(uint32_t); }
static constexpr size_t locate_smem_bytes(int block)
{
  return VGN_SMEM_STACK ? (size_t)kStackSize * block * sizeof(uint32_t) : 0;
}

// Opt a kernel in to more than 48 KiB of dynamic shared memory, once per (kernel, device).
template <typename Kernel>
static cudaError_t allow_smem(Kernel kernel, size_t bytes)
{
  static std::mutex m;
  static std::vector<std::pair<const void *, int>> done;
  if (bytes <= 48u * 1024u) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const auto key = std::make_pair(reinterpret_cast<const void *>(kernel), dev);
  std::lock_guard<std::mutex> lock(m);
  for (const auto &k : done)
    if (k == key) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.push_back(key);
  return e;
}

static inline unsigned grid_for(int64_t n, int block, int max_blocks)
{
  int64_t b = (n + block - 1) / block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

// The `sections` and `booleans` kernel sets instantiate one launch shape per kernel family
// (every variant number maps to it; results do not depend on the launch shape): with every
// shape, their units compiled for six and seven minutes.
#define VGN_ONE_LAUNCH_SHAPE (VGN_SECTIONS || VGN_BOOLEANS)

// Launch-shape variants of the step kernel (threads per block, minimum
// resident blocks per SM -> register cap); the autotuner picks one per geometry.
struct StepVariant {
  int block, minb;
};
static constexpr StepVariant kStepVariants[] = {{256, 2}, {256, 3}, {128, 6}, {256, 4}, {128, 5}, {128, 4}};
static constexpr int kNumStepVariants        = sizeof(kStepVariants) / sizeof(kStepVariants[0]);


template <bool MIXED, int BLOCK, int MINB>
static void launch_step_v(const GeomView &g, const StepArgs &a, cudaStream_t s)
{
  // grid-stride over tracks; enough blocks to fill every SM several times over
  const unsigned grid = grid_for(a.n, BLOCK, a.max_blocks * (256 / BLOCK));
  if (allow_smem(dev::step_kernel<MIXED, BLOCK, MINB>, step_smem_bytes(BLOCK)) != cudaSuccess) return;
  dev::step_kernel<MIXED, BLOCK, MINB><<<grid, BLOCK, step_smem_bytes(BLOCK), s>>>(
      g, a.n, a.px, a.py, a.pz, a.dx, a.dy, a.dz, a.slimit, a.in, a.out, a.step, a.reloc, a.perm);
}

// Variants of the mixed form with block-wide grouping (step_kernel_grouped), after the
// kStepVariants: shared memory decides the resident blocks (128 threads: 43 KiB per block,
// 256 threads: 85 KiB).
static constexpr StepVariant kGroupedVariants[] = {{128, 5}, {128, 4}, {256, 2}};
static constexpr int kNumGroupedVariants        = sizeof(kGroupedVariants) / sizeof(kGroupedVariants[0]);

int step_variant_count(bool mixed) { return kNumStepVariants + (mixed ? kNumGroupedVariants : 0); }
int multi_variant_count() { return kNumStepVariants; }

template <int BLOCK, int MINB>
static void launch_step_grouped(const GeomView &g, const StepArgs &a, cudaStream_t s)
{
#if !VGN_SMEM_STACK  // the grouping keeps its queues in shared memory: plain mixed step instead
  launch_step_v<true, BLOCK, MINB>(g, a, s);
#else
  const size_t smem   = dev::GroupLayout<BLOCK>::kBytes;
  const unsigned grid = grid_for(a.n, BLOCK, a.max_blocks * (256 / BLOCK));
  if (allow_smem(dev::step_kernel_grouped<BLOCK, MINB>, smem) != cudaSuccess) return;
  dev::step_kernel_grouped<BLOCK, MINB><<<grid, BLOCK, smem, s>>>(g, a.n, a.px, a.py, a.pz, a.dx, a.dy, a.dz,
                                                                  a.slimit, a.in, a.out, a.step, a.reloc, a.perm);
#endif
}

template <bool MIXED>
static void launch_step_m(const GeomView &g, const StepArgs &a, int variant, cudaStream_t s)
{
#if VGN_ONE_LAUNCH_SHAPE  // one launch shape per kernel family keeps this set's build short
  if (MIXED && variant >= kNumStepVariants)
    launch_step_grouped<128, 4>(g, a, s);
  else
    launch_step_v<MIXED, 128, 4>(g, a, s);
#else
  if (MIXED) {
    switch (variant) {
    case 6: launch_step_grouped<128, 5>(g, a, s); return;
    case 7: launch_step_grouped<128, 4>(g, a, s); return;
    case 8: launch_step_grouped<256, 2>(g, a, s); return;
    default: break;
    }
  }
  switch (variant) {
  case 1: launch_step_v<MIXED, 256, 3>(g, a, s); break;
  case 2: launch_step_v<MIXED, 128, 6>(g, a, s); break;
  case 3: launch_step_v<MIXED, 256, 4>(g, a, s); break;
  case 4: launch_step_v<MIXED, 128, 5>(g, a, s); break;
  case 5: launch_step_v<MIXED, 128, 4>(g, a, s); break;
  default: launch_step_v<MIXED, 256, 2>(g, a, s); break;
  }
#endif
}

// The safety runs as its own pass, before the step (which may overwrite the input states when
// out == in): fused into the step kernel it shares one register budget and one instruction
// footprint with the step traversal and the relocation, which measured slower than the two
// passes together.  Its visit order is its own when the caller binned tracks by position
// alone (the safety does not depend on the direction), else the step's.
static void launch_safety_pass(const GeomView &g, const StepArgs &a, bool mixed, cudaStream_t s)
{
  const unsigned grid = grid_for(a.n, dev::kSafetyBlock, a.max_blocks * (256 / dev::kSafetyBlock));
  if (mixed)
    dev::safety_kernel<true><<<grid, dev::kSafetyBlock, dev::kSafetySmemBytes, s>>>(g, a.n, a.px, a.py, a.pz, a.in, a.safety,
                                                                         a.perm_safety ? a.perm_safety : a.perm, 1);
  else
    dev::safety_kernel<false><<<grid, dev::kSafetyBlock, 0, s>>>(g, a.n, a.px, a.py, a.pz, a.in, a.safety,
                                                                  a.perm_safety ? a.perm_safety : a.perm, 1);
}

cudaError_t launch_safety_only(const GeomView &g, const StepArgs &a, bool mixed, cudaStream_t s)
{
  launch_safety_pass(g, a, mixed, s);
  return cudaGetLastError();
}

cudaError_t launch_step(const GeomView &g, const StepArgs &a, bool mixed, int variant, cudaStream_t s)
{
  if (a.safety) launch_safety_pass(g, a, mixed, s);
  if (mixed)
    launch_step_m<true>(g, a, variant, s);
  else
    launch_step_m<false>(g, a, variant, s);
  return cudaGetLastError();
}

template <bool MIXED, int BLOCK, int MINB>
static void launch_multi_v(const JobTable &jt, uint32_t *queue, int reloc, int num_sms, cudaStream_t s)
{
  // persistent: as many blocks as the variant keeps resident on every SM
  const unsigned grid = (unsigned)(num_sms * MINB);
  if (allow_smem(dev::multi_step_kernel<MIXED, BLOCK, MINB>, step_smem_bytes(BLOCK)) != cudaSuccess) return;
  dev::multi_step_kernel<MIXED, BLOCK, MINB><<<grid, BLOCK, step_smem_bytes(BLOCK), s>>>(jt, queue, reloc);
}

template <bool MIXED>
static void launch_multi_m(const JobTable &jt, uint32_t *queue, int reloc, int num_sms, int variant, cudaStream_t s)
{
#if VGN_ONE_LAUNCH_SHAPE
  (void)variant;
  launch_multi_v<MIXED, 128, 4>(jt, queue, reloc, num_sms, s);
#else
  switch (variant) {
  case 1: launch_multi_v<MIXED, 256, 3>(jt, queue, reloc, num_sms, s); break;
  case 2: launch_multi_v<MIXED, 128, 6>(jt, queue, reloc, num_sms, s); break;
  case 3: launch_multi_v<MIXED, 256, 4>(jt, queue, reloc, num_sms, s); break;
  case 4: launch_multi_v<MIXED, 128, 5>(jt, queue, reloc, num_sms, s); break;
  case 5: launch_multi_v<MIXED, 128, 4>(jt, queue, reloc, num_sms, s); break;
  default: launch_multi_v<MIXED, 256, 2>(jt, queue, reloc, num_sms, s); break;
  }
#endif
}

cudaError_t launch_multi_step(const JobTable &jt, uint32_t *queue, bool mixed, int reloc, int num_sms, int variant,
                              cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(queue, 0, 2 * sizeof(uint32_t), s);  // step and safety queues
  if (e != cudaSuccess) return e;
  bool any_safety = false;
  for (int k = 0; k < jt.n_jobs; ++k) any_safety = any_safety || jt.job[k].safety != nullptr;
  if (any_safety) {  // before the step, which may overwrite the input states
    const unsigned grid = (unsigned)(num_sms * 6);
    if (mixed)
      dev::multi_safety_kernel<true><<<grid, dev::kSafetyBlock, dev::kSafetySmemBytes, s>>>(jt, queue + 1);
    else
      dev::multi_safety_kernel<false><<<grid, dev::kSafetyBlock, 0, s>>>(jt, queue + 1);
  }
  if (mixed)
    launch_multi_m<true>(jt, queue, reloc, num_sms, variant, s);
  else
    launch_multi_m<false>(jt, queue, reloc, num_sms, variant, s);
  return cudaGetLastError();
}

template <int BLOCK, int MINB>
static cudaError_t launch_walk_grouped(const GeomView &g, int64_t n, double *px, double *py, double *pz,
                                       const double *dx, const double *dy, const double *dz, const double *slimit,
                                       vgn_state *state, int max_steps, int32_t *nsteps, const uint32_t *perm,
                                       int max_blocks, cudaStream_t s)
{
#if VGN_SMEM_STACK
  const unsigned grid = grid_for(n, dev::kWalkChunk * BLOCK, max_blocks);
  const size_t smem   = dev::GroupLayout<BLOCK>::kBytes;
  cudaError_t e       = allow_smem(dev::walk_kernel_grouped<BLOCK, MINB>, smem);
  if (e != cudaSuccess) return e;
  dev::walk_kernel_grouped<BLOCK, MINB><<<grid, BLOCK, smem, s>>>(g, n, px, py, pz, dx, dy, dz, slimit, state,
                                                                 max_steps, nsteps, perm);
  return cudaGetLastError();
#else
  return cudaErrorNotSupported;
#endif
}

cudaError_t launch_walk(const GeomView &g, int64_t n, double *px, double *py, double *pz, const double *dx,
                        const double *dy, const double *dz, const double *slimit, vgn_state *state, int max_steps,
                        int32_t *nsteps, const uint32_t *perm, bool mixed, int variant, int max_blocks,
                        cudaStream_t s)
{
#if VGN_ONE_LAUNCH_SHAPE
  if (mixed && VGN_SMEM_STACK && variant >= kNumStepVariants)
    return launch_walk_grouped<128, 4>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps, nsteps, perm, max_blocks, s);
#else
  if (mixed && VGN_SMEM_STACK) {
    switch (variant) {
    case 6: return launch_walk_grouped<128, 5>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps, nsteps, perm, max_blocks, s);
    case 7: return launch_walk_grouped<128, 4>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps, nsteps, perm, max_blocks, s);
    case 8: return launch_walk_grouped<256, 2>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps, nsteps, perm, max_blocks, s);
    default: break;
    }
  }
#endif
  const int block     = 128;
  const unsigned grid = grid_for(n, block, max_blocks * 2);
  const size_t smem   = step_smem_bytes(block);
  if (mixed)
    dev::walk_kernel<true><<<grid, block, smem, s>>>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps, nsteps,
                                                     perm);
  else
    dev::walk_kernel<false><<<grid, block, smem, s>>>(g, n, px, py, pz, dx, dy, dz, slimit, state, max_steps,
                                                      nsteps, perm);
  return cudaGetLastError();
}

cudaError_t launch_safety(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          const vgn_state *in, double *safety, bool mixed, int max_blocks, cudaStream_t s)
{
  const unsigned grid = grid_for(n, dev::kSafetyBlock, max_blocks * (256 / dev::kSafetyBlock));
  if (mixed)
    dev::safety_kernel<true><<<grid, dev::kSafetyBlock, dev::kSafetySmemBytes, s>>>(g, n, px, py, pz, in, safety, nullptr, 0);
  else
    dev::safety_kernel<false><<<grid, dev::kSafetyBlock, 0, s>>>(g, n, px, py, pz, in, safety, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t launch_locate(const GeomView &g, int64_t n, const double *px, const double *py, const double *pz,
                          vgn_state *out, bool mixed, int max_blocks, cudaStream_t s)
{
  const int block     = 256;
  const unsigned grid = grid_for(n, block, max_blocks);
  if (mixed)
    dev::locate_kernel<true><<<grid, block, locate_smem_bytes(block), s>>>(g, n, px, py, pz, out);
  else
    dev::locate_kernel<false><<<grid, block, locate_smem_bytes(block), s>>>(g, n, px, py, pz, out);
  return cudaGetLastError();
}

cudaError_t launch_approach(const GeomView &g, int64_t n, const int32_t *lv, const double *px, const double *py,
                            const double *pz, const double *dx, const double *dy, const double *dz,
                            const int32_t *last, double *step, int max_blocks, cudaStream_t s)
{
  const int block     = 256;
  const unsigned grid = grid_for(n, block, max_blocks);
  dev::approach_kernel<<<grid, block, locate_smem_bytes(block), s>>>(g, n, lv, px, py, pz, dx, dy, dz, last, step);
  return cudaGetLastError();
}

cudaError_t launch_shape_fp64(int op, int type, const double *row, int64_t n, const double *px, const double *py,
                              const double *pz, const double *dx, const double *dy, const double *dz,
                              const double *step_max, double *out, int max_blocks, cudaStream_t s)
{
  const int block     = 256;
  const unsigned grid = grid_for(n, block, max_blocks);
  switch (op) {
  case VGN_OP_DISTANCE_TO_IN:
    dev::shape_kernel_fp64<VGN_OP_DISTANCE_TO_IN><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  case VGN_OP_DISTANCE_TO_OUT:
    dev::shape_kernel_fp64<VGN_OP_DISTANCE_TO_OUT><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  case VGN_OP_SAFETY_TO_IN:
    dev::shape_kernel_fp64<VGN_OP_SAFETY_TO_IN><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  case VGN_OP_SAFETY_TO_OUT:
    dev::shape_kernel_fp64<VGN_OP_SAFETY_TO_OUT><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  case VGN_OP_CONTAINS:
    dev::shape_kernel_fp64<VGN_OP_CONTAINS><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  default:
    dev::shape_kernel_fp64<VGN_OP_INSIDE><<<grid, block, 0, s>>>(type, row, n, px, py, pz, dx, dy, dz, step_max, out);
    break;
  }
  return cudaGetLastError();
}

}  // namespace VGN_KSET
}  // namespace vgn
